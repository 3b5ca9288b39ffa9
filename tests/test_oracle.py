"""The C oracle, pinned: against the literal transcription, the golden fixtures and hand-derived answers."""

from pathlib import Path

import numpy as np
import pytest

from compiler import workloads as wl
from oracle import api, literal

GOLDEN = Path(__file__).with_name("golden") / "advection_small.npz"


def _bits(a):
    return np.ascontiguousarray(a).view(np.int64)


@pytest.mark.parametrize("shape", [(1, 1, 1), (3, 5, 2), (7, 4, 6)])
def test_c_oracle_matches_literal_transcription(shape):
    U, V, W, dx, dy, dz = literal.fixture_inputs(*shape)
    for which in ("cdu", "cdv", "cdw"):
        want = literal.tendency(which, np.zeros_like(U), U, V, W, dx, dy, dz)
        got = api.momentum(which, np.zeros_like(U), U, V, W, dx, dy, dz, 1)
        assert np.array_equal(_bits(got), _bits(want))


def test_random_fields_match_literal_transcription():
    f = wl.reference_driver_fields(6, 5, 4, seed=9)
    g = f.geometry
    for which in ("cdu", "cdv", "cdw"):
        want = literal.tendency(which, np.zeros_like(f.U), f.U, f.V, f.W, g.dx, g.dy, g.dz)
        got = api.momentum(which, np.zeros_like(f.U), f.U, f.V, f.W, g.dx, g.dy, g.dz, 1)
        assert np.array_equal(_bits(got), _bits(want))


def test_golden_fixtures():
    z = np.load(GOLDEN)
    dx, dy, dz = z["spacing"]
    for which in ("cdu", "cdv", "cdw"):
        got = api.momentum(which, np.zeros_like(z["U"]), z["U"], z["V"], z["W"], dx, dy, dz, 1)
        assert np.array_equal(_bits(got), _bits(z[which]))
    ins = [z[f"h2_in{n}"] for n in range(6)]
    geo = wl.Geometry(12, 10, 6, halo=2)
    t = api.advection_step({"U": ins[0], "V": ins[1], "W": ins[2]}, geo.dx, geo.dy, geo.dz, 2, ins[3:])
    for n, name in enumerate(["U", "V", "W", "S0", "S1", "S2"]):
        assert np.array_equal(_bits(t[name]), _bits(z[f"h2_tend{n}"]))
        step = api.halo(api.euler(ins[n].copy(), t[name], 0.1, 2), 1 if n == 2 else 0, 2)
        assert np.array_equal(_bits(step), _bits(z[f"h2_euler{n}"]))


def test_constant_velocities_have_zero_tendency():
    geo = wl.Geometry(5, 4, 3, halo=1)
    U = np.full(geo.shape, 1.75)
    V = np.full(geo.shape, -0.5)
    W = np.full(geo.shape, 2.25)
    for which in ("cdu", "cdv", "cdw"):
        t = api.momentum(which, np.ones_like(U), U, V, W, 1.0, 1.0, 1.0, 1)
        assert (t[geo.interior()] == 0.0).all()


def test_linear_zonal_velocity_known_answer():
    """U = i, V = W = 0, dx = 1: flux form gives -2i, advective form -i, CDU = 0.5*(-2i - i) = -1.5i."""
    geo = wl.Geometry(6, 3, 3, halo=1)
    i = np.arange(geo.shape[2], dtype=np.float64)
    U = np.broadcast_to(i, geo.shape).copy()
    Z = np.zeros(geo.shape)
    t = api.momentum("cdu", np.zeros_like(U), U, Z, Z, 1.0, 1.0, 1.0, 1)
    assert np.array_equal(t[geo.interior()], np.broadcast_to(-1.5 * i[1:-1], (3, 3, 6)))


def test_scalar_form_known_answers():
    geo = wl.Geometry(5, 5, 5, halo=1)
    s = np.full(geo.shape, 3.0)
    Z = np.zeros(geo.shape)
    assert (api.scalar(np.ones_like(s), s, Z, Z, Z, 1.0, 1.0, 1.0, 1)[geo.interior()] == 0.0).all()
    # uniform flow carries a uniform scalar without change
    U = np.full(geo.shape, 2.0)
    assert (api.scalar(np.ones_like(s), s, U, U, U, 1.0, 1.0, 1.0, 1)[geo.interior()] == 0.0).all()


def test_boundary_fill_matches_host_recipe_and_is_periodic():
    geo = wl.Geometry(9, 7, 6, halo=2)
    rng = np.random.default_rng(0)
    for kind in (0, 1):
        a = rng.normal(size=geo.shape)
        got = api.halo(a.copy(), kind, 2)
        want = wl.fill_halo(a.copy(), kind, 2)
        assert np.array_equal(_bits(got), _bits(want))
        assert np.array_equal(got[:, :, :2], got[:, :, 9:11])
        assert np.array_equal(got[:, :2, :], got[:, 7:9, :])
        if kind == 1:
            assert (got[1] == 0).all() and (got[2 + 6 - 1] == 0).all()


def test_stencil_oracle_known_answers():
    n = 6
    shape = (n + 2, n + 2, n + 2)
    x = np.broadcast_to(np.arange(n + 2, dtype=np.float64), shape).copy()
    b = api.diffusion7(np.zeros(shape), x, 0.125, 1.0, 1.0, 1)
    assert np.array_equal(b[1:-1, 1:-1, 1:-1], x[1:-1, 1:-1, 1:-1])  # linear: zero laplacian
    q = x * x
    b = api.diffusion7(np.zeros(shape), q, 0.125, 1.0, 1.0, 1)
    assert np.array_equal(b[1:-1, 1:-1, 1:-1], q[1:-1, 1:-1, 1:-1] + 0.25)
    u = np.full((10, 12), 4.0)
    v = api.jacobi5(np.zeros_like(u), u, 1)
    assert (v[1:-1, 1:-1] == 4.0).all()
    ez, hx, hy = np.zeros((8, 8)), np.zeros((8, 8)), np.zeros((8, 8))
    api.yee2d(ez, hx, hy, 0.5, 0.7, 1)
    assert not ez.any() and not hx.any() and not hy.any()


def test_ensemble_shapes_are_seeded():
    a = wl.ensemble_shapes(64, seed=1)
    assert a == wl.ensemble_shapes(64, seed=1)
    assert all(nx in wl.ENSEMBLE_XY and ny in wl.ENSEMBLE_XY and nz in wl.ENSEMBLE_Z for nx, ny, nz in a)
