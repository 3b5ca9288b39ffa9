"""ctypes front of the C oracle (test infrastructure only).

Arrays are numpy float64 of shape (nz+2h, ny+2h, nx+2h) in C order, which is
the Fortran column-major (nx+2h, ny+2h, nz+2h) layout of the reference.
"""

from __future__ import annotations

import ctypes
from functools import lru_cache

import numpy as np

from . import build as _build

_D = ctypes.c_double
_I = ctypes.c_int64
_P = ctypes.c_void_p


@lru_cache(maxsize=1)
def lib() -> ctypes.CDLL:
    handle = ctypes.CDLL(str(_build.build()))
    for name in ("orc_cdu", "orc_cdv", "orc_cdw"):
        getattr(handle, name).argtypes = [_P, _P, _P, _P, _D, _D, _D, _I, _I, _I, _I]
    handle.orc_scalar.argtypes = [_P, _P, _P, _P, _P, _D, _D, _D, _I, _I, _I, _I]
    handle.orc_halo.argtypes = [_P, ctypes.c_int, _I, _I, _I, _I]
    handle.orc_euler.argtypes = [_P, _P, _D, _I, _I, _I, _I]
    handle.orc_interior_sum.argtypes = [_P, _I, _I, _I, _I]
    handle.orc_interior_sum.restype = _D
    handle.orc_threads.restype = ctypes.c_int
    handle.orc_set_threads.argtypes = [ctypes.c_int]
    handle.orc_diffusion7.argtypes = [_P, _P, _D, _D, _D, _I, _I, _I, _I]
    handle.orc_jacobi5.argtypes = [_P, _P, _I, _I, _I]
    handle.orc_yee2d.argtypes = [_P, _P, _P, _D, _D, _I, _I, _I]
    return handle


def _ptr(a: np.ndarray) -> int:
    if a.dtype != np.float64 or not a.flags.c_contiguous:
        raise ValueError("oracle arrays must be C-contiguous float64")
    return a.ctypes.data


def _geometry(a: np.ndarray, h: int):
    nz, ny, nx = (s - 2 * h for s in a.shape)
    return nx, ny, nz


def momentum(which: str, out, U, V, W, dx, dy, dz, h):
    nx, ny, nz = _geometry(U, h)
    getattr(lib(), "orc_" + which)(_ptr(out), _ptr(U), _ptr(V), _ptr(W), dx, dy, dz, nx, ny, nz, h)
    return out


def scalar(out, s, U, V, W, dx, dy, dz, h):
    nx, ny, nz = _geometry(U, h)
    lib().orc_scalar(_ptr(out), _ptr(s), _ptr(U), _ptr(V), _ptr(W), dx, dy, dz, nx, ny, nz, h)
    return out


def halo(f, kind, h):
    nx, ny, nz = _geometry(f, h)
    lib().orc_halo(_ptr(f), int(kind), nx, ny, nz, h)
    return f


def euler(f, ft, dt, h):
    nx, ny, nz = _geometry(f, h)
    lib().orc_euler(_ptr(f), _ptr(ft), dt, nx, ny, nz, h)
    return f


def interior_sum(f, h) -> float:
    nx, ny, nz = _geometry(f, h)
    return lib().orc_interior_sum(_ptr(f), nx, ny, nz, h)


def threads() -> int:
    return lib().orc_threads()


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


def diffusion7(b, a, dt, nu, dx, h):
    nx, ny, nz = _geometry(a, h)
    lib().orc_diffusion7(_ptr(b), _ptr(a), dt, nu, dx, nx, ny, nz, h)
    return b


def jacobi5(v, u, h):
    ny, nx = (s - 2 * h for s in u.shape)
    lib().orc_jacobi5(_ptr(v), _ptr(u), nx, ny, h)
    return v


def yee2d(ez, hx, hy, ch, ce, h):
    ny, nx = (s - 2 * h for s in ez.shape)
    lib().orc_yee2d(_ptr(ez), _ptr(hx), _ptr(hy), ch, ce, nx, ny, h)


def advection_step(fields: dict, dx, dy, dz, h, scalars=(), out=None):
    """Tendencies of one step: U2, V2, W2 and one tendency per scalar.

    ``out`` (a dict with keys U, V, W, S0, ...) receives them when given; new
    zero-filled arrays are made otherwise.
    """
    U, V, W = fields["U"], fields["V"], fields["W"]
    if out is None:
        out = {name: np.zeros_like(U) for name in ("U", "V", "W", *[f"S{n}" for n in range(len(scalars))])}
    for name, which in (("U", "cdu"), ("V", "cdv"), ("W", "cdw")):
        momentum(which, out[name], U, V, W, dx, dy, dz, h)
    for n, s in enumerate(scalars):
        scalar(out[f"S{n}"], s, U, V, W, dx, dy, dz, h)
    return out
