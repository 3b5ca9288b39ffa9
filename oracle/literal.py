"""Literal, loop-by-loop Python transcription of the reference's advection procedures.

TEST INFRASTRUCTURE ONLY. This is the second, independent restatement of the
reference arithmetic. It follows the Fortran source statement by statement:
1-based indices with one ghost layer, the four calls of CDU in order (including
the dead ``set``), and every expression grouped exactly as written, evaluated
left to right. Python floats are IEEE binary64 with no contraction, so its
results are comparable bit for bit with the C oracle (advection_oracle.c, built
with -ffp-contract=off). It runs in pure Python loops and is meant for grids of
a few thousand points.

Sources followed:
  benchmarks/cdu/src/cdu.f90:12-27 (set), :30-45 (multiply), :48-76 (CDUdiv),
  :79-106 (CDUadv), :113-133 (CDU);
  compiler/tests/fixtures/stencils/cvd.f90:44-125 (CDVdiv, CDVadv, CDV);
  compiler/tests/fixtures/stencils/cdw.f90:44-125 (CDWdiv, CDWadv, CDW);
  compiler/tests/fixtures/stencils/cdu_main.f90:38-50 (deterministic inputs).
"""

from __future__ import annotations

import math

import numpy as np


class F3:
    """A Fortran array ``A(1:n1, 1:n2, 1:n3)`` over a column-major numpy buffer."""

    def __init__(self, data: np.ndarray):
        self.a = data  # shape (n3, n2, n1) in C order == column-major (n1, n2, n3)

    def __call__(self, i, j, k):
        return float(self.a[k - 1, j - 1, i - 1])

    def set(self, i, j, k, value):
        self.a[k - 1, j - 1, i - 1] = value


def _set(arr, val, n1, n2, n3):
    for k in range(2, n3 + 2):
        for j in range(2, n2 + 2):
            for i in range(2, n1 + 2):
                arr.set(i, j, k, val)


def _multiply(arr, val, n1, n2, n3):
    for k in range(2, n3 + 2):
        for j in range(2, n2 + 2):
            for i in range(2, n1 + 2):
                arr.set(i, j, k, arr(i, j, k) * val)


def _cdu_div(U2, U, V, W, dxmin, dymin, dzmin, n1, n2, n3):
    Ax = 0.25 / dxmin
    Ay = 0.25 / dymin
    Az = 0.25 / dzmin
    for k in range(2, n3 + 2):
        for j in range(2, n2 + 2):
            for i in range(2, n1 + 2):
                U2.set(i, j, k, -((Ax * (U(i + 1, j, k) + U(i, j, k)) * (U(i + 1, j, k) + U(i, j, k))
                                   - Ax * (U(i, j, k) + U(i - 1, j, k)) * (U(i, j, k) + U(i - 1, j, k)))
                                  + (Ay * (U(i, j + 1, k) + U(i, j, k)) * (V(i + 1, j, k) + V(i, j, k))
                                     - Ay * (U(i, j, k) + U(i, j - 1, k)) * (V(i + 1, j - 1, k) + V(i, j - 1, k)))
                                  + (Az * (U(i, j, k + 1) + U(i, j, k)) * (W(i + 1, j, k) + W(i, j, k))
                                     - Az * (U(i, j, k) + U(i, j, k - 1)) * (W(i + 1, j, k - 1) + W(i, j, k - 1)))))


def _cdu_adv(U2, U, V, W, dxmin, dymin, dzmin, n1, n2, n3):
    Ax = 0.5 / dxmin
    Ay = 0.125 / dymin
    Az = 0.125 / dzmin
    for k in range(2, n3 + 2):
        for j in range(2, n2 + 2):
            for i in range(2, n1 + 2):
                Vadv = (V(i, j, k) + V(i + 1, j, k) + V(i, j - 1, k) + V(i + 1, j - 1, k))
                Wadv = (W(i, j, k) + W(i + 1, j, k) + W(i, j, k - 1) + W(i + 1, j, k - 1))
                U2.set(i, j, k, U2(i, j, k)
                       - (Ax * (U(i + 1, j, k) - U(i - 1, j, k)) * U(i, j, k)
                          + Ay * (U(i, j + 1, k) - U(i, j - 1, k)) * Vadv
                          + Az * (U(i, j, k + 1) - U(i, j, k - 1)) * Wadv))


def _cdv_div(V2, U, V, W, dxmin, dymin, dzmin, n1, n2, n3):
    Ax = 0.25 / dxmin
    Ay = 0.25 / dymin
    Az = 0.25 / dzmin
    for k in range(2, n3 + 2):
        for j in range(2, n2 + 2):
            for i in range(2, n1 + 2):
                V2.set(i, j, k, -((Ay * (V(i, j + 1, k) + V(i, j, k)) * (V(i, j + 1, k) + V(i, j, k))
                                   - Ay * (V(i, j, k) + V(i, j - 1, k)) * (V(i, j, k) + V(i, j - 1, k)))
                                  + (Ax * (V(i + 1, j, k) + V(i, j, k)) * (U(i, j + 1, k) + U(i, j, k))
                                     - Ax * (V(i, j, k) + V(i - 1, j, k)) * (U(i - 1, j + 1, k) + U(i - 1, j, k)))
                                  + (Az * (V(i, j, k + 1) + V(i, j, k)) * (W(i, j + 1, k) + W(i, j, k))
                                     - Az * (V(i, j, k) + V(i, j, k - 1)) * (W(i, j + 1, k - 1) + W(i, j, k - 1)))))


def _cdv_adv(V2, U, V, W, dxmin, dymin, dzmin, n1, n2, n3):
    Ax = 0.125 / dxmin
    Ay = 0.5 / dymin
    Az = 0.125 / dzmin
    for k in range(2, n3 + 2):
        for j in range(2, n2 + 2):
            for i in range(2, n1 + 2):
                Uadv = (U(i, j, k) + U(i, j + 1, k) + U(i - 1, j, k) + U(i - 1, j + 1, k))
                Wadv = (W(i, j, k) + W(i, j + 1, k) + W(i, j, k - 1) + W(i, j + 1, k - 1))
                V2.set(i, j, k, V2(i, j, k)
                       - (Ax * (V(i + 1, j, k) - V(i - 1, j, k)) * Uadv
                          + Ay * (V(i, j + 1, k) - V(i, j - 1, k)) * V(i, j, k)
                          + Az * (V(i, j, k + 1) - V(i, j, k - 1)) * Wadv))


def _cdw_div(W2, U, V, W, dxmin, dymin, dzmin, n1, n2, n3):
    Ax = 0.25 / dxmin
    Ay = 0.25 / dymin
    Az = 0.25 / dzmin
    for k in range(2, n3 + 2):
        for j in range(2, n2 + 2):
            for i in range(2, n1 + 2):
                W2.set(i, j, k, -((Az * (W(i, j, k + 1) + W(i, j, k)) * (W(i, j, k + 1) + W(i, j, k))
                                   - Az * (W(i, j, k) + W(i, j, k - 1)) * (W(i, j, k) + W(i, j, k - 1)))
                                  + (Ay * (W(i, j + 1, k) + W(i, j, k)) * (V(i, j, k + 1) + V(i, j, k))
                                     - Ay * (W(i, j, k) + W(i, j - 1, k)) * (V(i, j - 1, k) + V(i, j - 1, k + 1)))
                                  + (Ax * (W(i + 1, j, k) + W(i, j, k)) * (U(i, j, k + 1) + U(i, j, k))
                                     - Ax * (W(i, j, k) + W(i - 1, j, k)) * (U(i - 1, j, k + 1) + U(i - 1, j, k)))))


def _cdw_adv(W2, U, V, W, dxmin, dymin, dzmin, n1, n2, n3):
    Ax = 0.125 / dxmin
    Ay = 0.125 / dymin
    Az = 0.5 / dzmin
    for k in range(2, n3 + 2):
        for j in range(2, n2 + 2):
            for i in range(2, n1 + 2):
                Uadv = (U(i, j, k) + U(i, j, k + 1) + U(i - 1, j, k) + U(i - 1, j, k + 1))
                Vadv = (V(i, j, k) + V(i, j, k + 1) + V(i, j - 1, k) + V(i, j - 1, k + 1))
                W2.set(i, j, k, W2(i, j, k)
                       - (Ax * (W(i + 1, j, k) - W(i - 1, j, k)) * Uadv
                          + Ay * (W(i, j + 1, k) - W(i, j - 1, k)) * Vadv
                          + Az * (W(i, j, k + 1) - W(i, j, k - 1)) * W(i, j, k)))


_PROCEDURES = {"cdu": (_cdu_div, _cdu_adv), "cdv": (_cdv_div, _cdv_adv), "cdw": (_cdw_div, _cdw_adv)}


def tendency(which: str, out: np.ndarray, U: np.ndarray, V: np.ndarray, W: np.ndarray,
             dxmin: float, dymin: float, dzmin: float) -> np.ndarray:
    """CDU / CDV / CDW on arrays of shape (NZ+2, NY+2, NX+2) (C order == Fortran (NX+2, NY+2, NZ+2)).

    ``out`` is updated in place like the Fortran ``intent(out)`` dummy: its
    ghost layer keeps whatever it held.
    """
    div, adv = _PROCEDURES[which]
    n3, n2, n1 = (s - 2 for s in out.shape)
    a2, a, b, c = F3(out), F3(U), F3(V), F3(W)
    zero, half = 0.0, 0.5
    _set(a2, zero, n1, n2, n3)
    div(a2, a, b, c, dxmin, dymin, dzmin, n1, n2, n3)
    adv(a2, a, b, c, dxmin, dymin, dzmin, n1, n2, n3)
    _multiply(a2, half, n1, n2, n3)
    return out


def fixture_inputs(nx: int, ny: int, nz: int):
    """The deterministic sin/cos inputs of compiler/tests/fixtures/stencils/cdu_main.f90:38-50.

    Returns U, V, W of shape (NZ+2, NY+2, NX+2) and the spacings 1/N of :34-36.
    ``math.sin``/``math.cos`` are the platform libm's; the values are inputs only.
    """
    U = np.empty((nz + 2, ny + 2, nx + 2))
    V = np.empty_like(U)
    W = np.empty_like(U)
    for k in range(1, nz + 3):
        for j in range(1, ny + 3):
            for i in range(1, nx + 3):
                U[k - 1, j - 1, i - 1] = math.sin(float(i) * 0.3) * math.cos(float(j) * 0.5) * (1.0 + 0.1 * float(k))
                V[k - 1, j - 1, i - 1] = math.cos(float(i) * 0.7) * math.sin(float(k) * 0.4) * (1.0 + 0.1 * float(j))
                W[k - 1, j - 1, i - 1] = math.sin(float(j) * 0.6 + float(k) * 0.2)
    return U, V, W, 1.0 / float(nx), 1.0 / float(ny), 1.0 / float(nz)
