// Per-point arithmetic of the advection templates, grouped exactly as the
// reference sources write it (left to right, parentheses kept). Built with
// --fmad=false, each expression rounds like the Fortran control and the C
// oracle, so results are bit-identical.
//
//   cdu_point: benchmarks/cdu/src/cdu.f90:66-71 (CDUdiv) then :96-101 (CDUadv)
//              then * 0.5 (:39, multiply by `half` from CDU :124-132)
//   cdv_point: compiler/tests/fixtures/stencils/cvd.f90:61-66 then :89-94, * 0.5
//   cdw_point: compiler/tests/fixtures/stencils/cdw.f90:61-66 then :89-94, * 0.5
//   scalar_point: this project's centred flux form (no reference source exists
//              in the mount for scalar advection).
#pragma once
#include <cstdint>

namespace f2c {

struct Coefficients {
    double Ax, Ay, Az;    // 0.25/d: every *div procedure
    double Bux, Buy, Buz; // CDUadv: 0.5/dx, 0.125/dy, 0.125/dz
    double Bvx, Bvy, Bvz; // CDVadv: 0.125/dx, 0.5/dy, 0.125/dz
    double Bwx, Bwy, Bwz; // CDWadv: 0.125/dx, 0.125/dy, 0.5/dz
    double Sx, Sy, Sz;    // scalar flux: 0.5/d
};

// F(a, di, dj, dk) reads array a at the point offset by (di, dj, dk).
// *_DIV is the flux-form procedure (it overwrites the output), *_ADV(prev)
// subtracts the advective form from the value `prev` (the procedure's
// read-modify-write of the output), *_POINT is the whole procedure: DIV, then
// ADV of it, then the multiplication by one half.
#define F2C_CDU_DIV(F, C)                                                                                           \
    (-(((C).Ax * (F(U, 1, 0, 0) + F(U, 0, 0, 0)) * (F(U, 1, 0, 0) + F(U, 0, 0, 0)) -                                \
        (C).Ax * (F(U, 0, 0, 0) + F(U, -1, 0, 0)) * (F(U, 0, 0, 0) + F(U, -1, 0, 0))) +                             \
       ((C).Ay * (F(U, 0, 1, 0) + F(U, 0, 0, 0)) * (F(V, 1, 0, 0) + F(V, 0, 0, 0)) -                                \
        (C).Ay * (F(U, 0, 0, 0) + F(U, 0, -1, 0)) * (F(V, 1, -1, 0) + F(V, 0, -1, 0))) +                            \
       ((C).Az * (F(U, 0, 0, 1) + F(U, 0, 0, 0)) * (F(W, 1, 0, 0) + F(W, 0, 0, 0)) -                                \
        (C).Az * (F(U, 0, 0, 0) + F(U, 0, 0, -1)) * (F(W, 1, 0, -1) + F(W, 0, 0, -1)))))

#define F2C_CDU_ADV(F, C, prev)                                                                                     \
    ([&]() -> double {                                                                                              \
        const double Vadv = (F(V, 0, 0, 0) + F(V, 1, 0, 0) + F(V, 0, -1, 0) + F(V, 1, -1, 0));                      \
        const double Wadv = (F(W, 0, 0, 0) + F(W, 1, 0, 0) + F(W, 0, 0, -1) + F(W, 1, 0, -1));                      \
        return (prev) - ((C).Bux * (F(U, 1, 0, 0) - F(U, -1, 0, 0)) * F(U, 0, 0, 0) +                               \
                         (C).Buy * (F(U, 0, 1, 0) - F(U, 0, -1, 0)) * Vadv +                                        \
                         (C).Buz * (F(U, 0, 0, 1) - F(U, 0, 0, -1)) * Wadv);                                        \
    }())

#define F2C_CDV_DIV(F, C)                                                                                           \
    (-(((C).Ay * (F(V, 0, 1, 0) + F(V, 0, 0, 0)) * (F(V, 0, 1, 0) + F(V, 0, 0, 0)) -                                \
        (C).Ay * (F(V, 0, 0, 0) + F(V, 0, -1, 0)) * (F(V, 0, 0, 0) + F(V, 0, -1, 0))) +                             \
       ((C).Ax * (F(V, 1, 0, 0) + F(V, 0, 0, 0)) * (F(U, 0, 1, 0) + F(U, 0, 0, 0)) -                                \
        (C).Ax * (F(V, 0, 0, 0) + F(V, -1, 0, 0)) * (F(U, -1, 1, 0) + F(U, -1, 0, 0))) +                            \
       ((C).Az * (F(V, 0, 0, 1) + F(V, 0, 0, 0)) * (F(W, 0, 1, 0) + F(W, 0, 0, 0)) -                                \
        (C).Az * (F(V, 0, 0, 0) + F(V, 0, 0, -1)) * (F(W, 0, 1, -1) + F(W, 0, 0, -1)))))

#define F2C_CDV_ADV(F, C, prev)                                                                                     \
    ([&]() -> double {                                                                                              \
        const double Uadv = (F(U, 0, 0, 0) + F(U, 0, 1, 0) + F(U, -1, 0, 0) + F(U, -1, 1, 0));                      \
        const double Wadv = (F(W, 0, 0, 0) + F(W, 0, 1, 0) + F(W, 0, 0, -1) + F(W, 0, 1, -1));                      \
        return (prev) - ((C).Bvx * (F(V, 1, 0, 0) - F(V, -1, 0, 0)) * Uadv +                                        \
                         (C).Bvy * (F(V, 0, 1, 0) - F(V, 0, -1, 0)) * F(V, 0, 0, 0) +                               \
                         (C).Bvz * (F(V, 0, 0, 1) - F(V, 0, 0, -1)) * Wadv);                                        \
    }())

#define F2C_CDW_DIV(F, C)                                                                                           \
    (-(((C).Az * (F(W, 0, 0, 1) + F(W, 0, 0, 0)) * (F(W, 0, 0, 1) + F(W, 0, 0, 0)) -                                \
        (C).Az * (F(W, 0, 0, 0) + F(W, 0, 0, -1)) * (F(W, 0, 0, 0) + F(W, 0, 0, -1))) +                             \
       ((C).Ay * (F(W, 0, 1, 0) + F(W, 0, 0, 0)) * (F(V, 0, 0, 1) + F(V, 0, 0, 0)) -                                \
        (C).Ay * (F(W, 0, 0, 0) + F(W, 0, -1, 0)) * (F(V, 0, -1, 0) + F(V, 0, -1, 1))) +                            \
       ((C).Ax * (F(W, 1, 0, 0) + F(W, 0, 0, 0)) * (F(U, 0, 0, 1) + F(U, 0, 0, 0)) -                                \
        (C).Ax * (F(W, 0, 0, 0) + F(W, -1, 0, 0)) * (F(U, -1, 0, 1) + F(U, -1, 0, 0)))))

#define F2C_CDW_ADV(F, C, prev)                                                                                     \
    ([&]() -> double {                                                                                              \
        const double Uadv = (F(U, 0, 0, 0) + F(U, 0, 0, 1) + F(U, -1, 0, 0) + F(U, -1, 0, 1));                      \
        const double Vadv = (F(V, 0, 0, 0) + F(V, 0, 0, 1) + F(V, 0, -1, 0) + F(V, 0, -1, 1));                      \
        return (prev) - ((C).Bwx * (F(W, 1, 0, 0) - F(W, -1, 0, 0)) * Uadv +                                        \
                         (C).Bwy * (F(W, 0, 1, 0) - F(W, 0, -1, 0)) * Vadv +                                        \
                         (C).Bwz * (F(W, 0, 0, 1) - F(W, 0, 0, -1)) * F(W, 0, 0, 0));                               \
    }())

#define F2C_CDU_POINT(F, C) (F2C_CDU_ADV(F, C, F2C_CDU_DIV(F, C)) * 0.5)
#define F2C_CDV_POINT(F, C) (F2C_CDV_ADV(F, C, F2C_CDV_DIV(F, C)) * 0.5)
#define F2C_CDW_POINT(F, C) (F2C_CDW_ADV(F, C, F2C_CDW_DIV(F, C)) * 0.5)

// Scalar S advected by U, V, W (face fluxes shareable between neighbours).
#define F2C_SCALAR_POINT(F, S, C)                                                                                   \
    ([&]() -> double {                                                                                              \
        const double c = F(S, 0, 0, 0);                                                                             \
        const double fe = ((C).Sx * F(U, 0, 0, 0)) * (F(S, 1, 0, 0) + c);                                           \
        const double fw = ((C).Sx * F(U, -1, 0, 0)) * (c + F(S, -1, 0, 0));                                         \
        const double fn = ((C).Sy * F(V, 0, 0, 0)) * (F(S, 0, 1, 0) + c);                                           \
        const double fs = ((C).Sy * F(V, 0, -1, 0)) * (c + F(S, 0, -1, 0));                                         \
        const double ft = ((C).Sz * F(W, 0, 0, 0)) * (F(S, 0, 0, 1) + c);                                           \
        const double fb = ((C).Sz * F(W, 0, 0, -1)) * (c + F(S, 0, 0, -1));                                         \
        return -(((fe - fw) + (fn - fs)) + (ft - fb));                                                              \
    }())

// Coefficients of the factored (fast-fp) form of the same tendencies
// (advection_fast.cuh). With A = 0.25/d per direction, the reference's
// skew-symmetric average -(1/2)(div + adv) of each momentum component regroups,
// in exact arithmetic, into one product per direction: the direction along the
// component ("diagonal") carries -A/2 and the two others ("cross") -A/4.
// Scalars use 0.5/d. In ADVANCE mode every coefficient is multiplied by dt, so
// that out = in + dt*tendency costs no extra operation.
struct FastCoefficients {
    double gx, gy, gz;    // diagonal: -0.125/d (times dt)
    double cx, cy, cz;    // cross: -0.0625/d (times dt)
    double sx, sy, sz;    // scalar: 0.5/d (times dt)
};

inline FastCoefficients make_fast_coefficients(double dx, double dy, double dz, int advance, double dt) {
    const double t = advance ? dt : 1.0;
    FastCoefficients f;
    f.gx = -(0.125 / dx) * t; f.gy = -(0.125 / dy) * t; f.gz = -(0.125 / dz) * t;
    f.cx = -(0.0625 / dx) * t; f.cy = -(0.0625 / dy) * t; f.cz = -(0.0625 / dz) * t;
    f.sx = (0.5 / dx) * t; f.sy = (0.5 / dy) * t; f.sz = (0.5 / dz) * t;
    return f;
}

inline Coefficients make_coefficients(double dx, double dy, double dz) {
    Coefficients c;
    c.Ax = 0.25 / dx; c.Ay = 0.25 / dy; c.Az = 0.25 / dz;
    c.Bux = 0.5 / dx; c.Buy = 0.125 / dy; c.Buz = 0.125 / dz;
    c.Bvx = 0.125 / dx; c.Bvy = 0.5 / dy; c.Bvz = 0.125 / dz;
    c.Bwx = 0.125 / dx; c.Bwy = 0.125 / dy; c.Bwz = 0.5 / dz;
    c.Sx = 0.5 / dx; c.Sy = 0.5 / dy; c.Sz = 0.5 / dz;
    return c;
}

} // namespace f2c
