"""The device evaluates van Genuchten saturation and Mualem relative
permeability with four powers per unsaturated cell instead of the nine of the
reference's formulas (src/materials/tdycharacteristiccurves.c:692-717 and the
Mualem branch at :468-485), using identities of the same bases.  This checks,
in FP64 on the CPU, that both forms agree to rounding over the parameter
ranges the workloads use, including nearly saturated and very dry states."""
import numpy as np


def vg_reference(m, alpha, Pc):
    n = 1.0 / (1.0 - m)
    x = Pc * alpha
    xn = x ** n
    op = 1.0 + xn
    Se = op ** (-m)
    dSe = -m * n * alpha * xn / (x * op ** (m + 1))
    d2Se = m * n * xn * op ** (-m - 2.0) * ((m * n + 1.0) * xn - n + 1) / (Pc * Pc)
    return Se, dSe, d2Se


def vg_identities(m, alpha, Pc):
    n = 1.0 / (1.0 - m)
    x = Pc * alpha
    xn = x ** n
    op = 1.0 + xn
    Se = op ** (-m)
    dSe = -m * n * alpha * xn * Se / (x * op)                           # op^(m+1) = op / Se
    d2Se = m * n * xn * (Se / (op * op)) * ((m * n + 1.0) * xn - n + 1) / (Pc * Pc)  # op^(-m-2) = Se / op^2
    return Se, dSe, d2Se


def mualem_reference(m, Se):
    so = Se ** (1 / m)
    tmp = (1 - so) ** m
    kr = np.sqrt(Se) * ((1 - tmp) * (1 - tmp))
    d = 0.5 * kr / Se + 2 * Se ** (1 / m - 0.5) * (1 - so) ** (m - 1) * (1 - (1 - so) ** m)
    return kr, d


def mualem_identities(m, Se):
    so = Se ** (1 / m)
    oms = 1 - so
    tmp = oms ** m
    sq = np.sqrt(Se)
    kr = sq * ((1 - tmp) * (1 - tmp))
    d = 0.5 * kr / Se + 2 * (so / sq) * (tmp / oms) * (1 - tmp)    # Se^(1/m-1/2) = so/sqrt(Se), oms^(m-1) = tmp/oms
    return kr, d


def rel(a, b):
    return np.max(np.abs(a - b) / np.maximum(np.abs(b), np.finfo(float).tiny))


def test_van_genuchten_identities():
    m = np.linspace(0.2, 0.6, 9)[:, None, None]
    alpha = np.logspace(-5, -3, 7)[None, :, None]
    Pc = np.logspace(-2, 6, 200)[None, None, :]  # from nearly saturated to very dry
    for a, b in zip(vg_identities(m, alpha, Pc), vg_reference(m, alpha, Pc)):
        assert rel(a, b) < 1e-13


def test_mualem_identities():
    m = np.linspace(0.2, 0.6, 9)[:, None]
    Se = np.concatenate([np.logspace(-8, -1, 100), 1.0 - np.logspace(-1, -12, 100)])[None, :]
    kr_a, d_a = mualem_identities(m, Se)
    kr_b, d_b = mualem_reference(m, Se)
    assert rel(kr_a, kr_b) < 1e-12
    assert rel(d_a, d_b) < 1e-12
