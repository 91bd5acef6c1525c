"""Mesh generators of the synthetic workloads (CPU only)."""
import numpy as np

from tdycore_gb300 import workloads as W


def _max_angles(xy, tris):
    P = xy[tris]
    a = np.linalg.norm(P[:, 1] - P[:, 2], axis=1)
    b = np.linalg.norm(P[:, 0] - P[:, 2], axis=1)
    c = np.linalg.norm(P[:, 0] - P[:, 1], axis=1)
    A = np.degrees(np.arccos(np.clip((b * b + c * c - a * a) / (2 * b * c), -1, 1)))
    B = np.degrees(np.arccos(np.clip((a * a + c * c - b * b) / (2 * a * c), -1, 1)))
    return np.maximum(np.maximum(A, B), 180.0 - A - B)


def test_delaunay_surface_has_no_hull_slivers():
    """Side points at the interior spacing and an h/4 margin keep the
    triangles along the sides well shaped; every point is used, triangles are
    counter-clockwise and tile the square."""
    for npts in (25, 2000, 20000):
        xy, tris = W.delaunay_surface(npts, 1000.0, 800.0, W._rng(30))
        assert len(np.unique(tris)) == xy.shape[0]
        P = xy[tris]
        cross = (P[:, 1, 0] - P[:, 0, 0]) * (P[:, 2, 1] - P[:, 0, 1]) - (P[:, 1, 1] - P[:, 0, 1]) * (P[:, 2, 0] - P[:, 0, 0])
        assert np.all(cross > 0)
        assert abs(0.5 * cross.sum() - 1000.0 * 800.0) < 1e-6 * 1000.0 * 800.0
        on_side = (np.isclose(xy[:, 0], 0) | np.isclose(xy[:, 0], 1000.0) | np.isclose(xy[:, 1], 0)
                   | np.isclose(xy[:, 1], 800.0))
        touches_side = on_side[tris].sum(axis=1) >= 2
        assert _max_angles(xy, tris)[touches_side].max() < 150.0


def test_random_spd_rotations_and_anisotropy():
    rng = np.random.default_rng(1)
    for rotation in ("full", "vertical"):
        K = W.random_spd(500, rng, rotation=rotation)
        assert np.allclose(K, np.transpose(K, (0, 2, 1)))
        assert np.all(np.linalg.eigvalsh(K) > 0)
        if rotation == "vertical":
            assert np.all(K[:, 0, 2] == 0) and np.all(K[:, 1, 2] == 0)
    K = W.random_spd(20000, rng, anisotropy_std=0.25)
    ev = np.log10(np.linalg.eigvalsh(K))
    assert abs(ev.mean() + 12.0) < 0.05 and abs(ev.std() - 1.0) < 0.05
    assert np.std(ev[:, 2] - ev[:, 0]) < 1.0


def test_workloads_are_seeded():
    """Every generator the bench uses is seeded: two builds give the same
    mesh, materials, boundary data and start, so both arms and every run see
    the same inputs."""
    import tdycore_gb300 as T
    from tdycore_gb300 import workloads as W

    def view(build):
        T.options_clear()
        t, U = build()
        t.setup(host_only=True)
        v = t.setup_view()
        t.destroy()
        return v, U

    builds = {
        "spe10_like": lambda: W.spe10_like(8, 7, 5, seed_offset=3)[:2],
        "batched_columns": lambda: W.batched_columns(12)[:2],
        "infiltration_prisms": lambda: W.infiltration_prisms(60, 4)[:2],
    }
    for name, build in builds.items():
        (v1, U1), (v2, U2) = view(build), view(build)
        assert np.array_equal(U1, U2), name
        for k, a in v1.items():
            if isinstance(a, np.ndarray):
                assert np.array_equal(a, v2[k]), (name, k)
            else:
                assert a == v2[k], (name, k)
