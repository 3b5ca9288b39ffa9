// Factored ("fast-fp") z-marching advection kernel for sm_103a.
//
// The reference's --fast-fp build (compiler/resident/build.py:22,66-67) trades
// the strict contract for FMA contraction. This kernel goes further in the same
// direction: it evaluates the same tendencies as the strict face-sharing kernel
// (advection_faces.cuh) through an algebraically regrouped form that spends
// about 80 floating-point operations per grid point (U, V, W and three
// scalars) where the reference grouping needs 126. GB300 issues FP64 at about
// two lane operations per clock per SM, so the FP64 instruction count is what
// bounds the step; everything else here (loads, shuffles, shared memory,
// integer work) runs on otherwise idle pipes. That includes the twelve plain
// products, which are computed on the integer pipes (pmul, soft_fp64.cuh; the
// same correctly rounded values), leaving 68 instructions per point on the
// FP64 pipe.
//
// Regrouping (exact in real arithmetic; A = 0.25/d per direction). For the U
// component of benchmarks/cdu/src/cdu.f90:66-71,96-101 with the final
// multiplication by one half (:39):
//   x: Ax[(Ue+U0)^2 - (U0+Uw)^2] + 2Ax(Ue-Uw)U0 = Ax (Ue-Uw)(Ue+Uw+4U0)
//   y: Ay[n vn - s vs] + (Ay/2)(n-s)(vn+vs)     = (Ay/2)[n(3vn+vs) - s(3vs+vn)]
// where n, s are U's north and south face sums (U(j+1)+U, U+U(j-1)) and vn, vs
// the V face sums at the same corners (V(i+1)+V at rows j and j-1); z is the y
// form with U's top/bottom face sums and W's. The advective coefficients of the
// reference (0.5/d along the component, 0.125/d across) are exactly 2A and A/2,
// and Un-Us = n-s, so the flux and advective forms share every face sum. V and
// W rotate the roles (compiler/tests/fixtures/stencils/{cvd,cdw}.f90:61-66,
// 89-94). The tendency is -(1/2) of the sum, so each direction is one product
// scaled by -A/2 (along the component) or -A/4 (across), accumulated by FMA.
//
// Scalars (this project's centred flux form, advection_point.cuh) regroup as
//   -sum_d [c0 (Se+S0) - cw (S0+Sw)] = S0*D - sum_d (c0 Se - cw Sw),
//   c = 0.5/d times the velocity at the face, D = sum_d (cw - c0),
// with D shared by all scalars: 7 FP64 instructions per scalar instead of 11.
//
// Each point's own face sums (six, U(j+1)+U etc.) and scaled velocities (three)
// are computed once and handed to the neighbours that need them: the x
// neighbour by a warp shuffle, the y neighbour through a shared-memory row
// exchange (an extra "edge" warp supplies the tile's south row and west
// column), the level above in registers carried up the z-march. Results differ
// from the reference's rounding by a few units in the last place of the
// intermediate sums (measured max relative error ~1e-15 of each field's
// maximum); the strict kernel stays the bit-exact default.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "advection_faces.cuh"
#include "advection_kernels.cuh"

namespace f2c {

constexpr int kFastTX = 32;        // points per tile along x (one warp)
constexpr int kFastKZ = 32;        // levels per z-chunk for large grids
constexpr int kFastSlots = 5;      // values exchanged per face row or column

// Shared exchange of one level, double-buffered: the north-face values of
// every row of the tile ([slot][row][lane], row 0 = the row south of the tile)
// and the east-face values of the column west of the tile ([slot][row]).
template <int TY>
struct FastSmem {
    static constexpr int SOUTH = kFastSlots * (TY + 1) * kFastTX;
    static constexpr int WEST = kFastSlots * TY;
    static constexpr int PER_BUFFER = SOUTH + WEST;
    static constexpr int doubles = 2 * PER_BUFFER;
};

template <int TY>
constexpr int fast_threads() { return kFastTX * (TY + 1); }

// CTAs per SM a tile height is compiled for by default: the register budget
// follows (96 registers a thread at four 5-warp or two 9-warp CTAs, more at
// one 17-warp CTA).
template <int TY>
constexpr int fast_ctas_per_sm() { return TY <= 4 ? 4 : (TY <= 8 ? 2 : 1); }

// Tile height of the single-instance launches, and the CTAs per SM their
// kernel is compiled for when the launch has at least kFastDeepCtas CTAs per
// SM of work (72 registers; the three-scalar step then spills about 240 bytes
// a thread, served by L1). More warps hide more of the FP64 and integer
// latencies of large grids; measured at 512 x 512 x 128 with three
// scalars, 8-row tiles took 4.10 ms at two CTAs per SM, 3.94 at three and 3.95
// at four (4-row tiles 4.06, 4.03 and 4.03 at four, six and eight; 16-row
// tiles 4.31 at one and 4.09 at two). Smaller launches keep two CTAs: at three
// the 64 uneven instances of the ensemble, launched one at a time, ran 6 %
// slower, and so did the serving ticks' batched steps.
constexpr int kFastTY = 8;
constexpr int kFastDeepCtasPerSM = 3;
constexpr int kFastDeepCtas = 8;

// p(3q + qn) - pn(3qn + q): one direction of a momentum component across its
// own axis, with p, pn the component's own face sums at the near and far face
// and q, qn the other velocity's face sums at the same faces.
__device__ __forceinline__ double cross_term(double p, double pn, double q, double qn) {
    const double a = __fma_rn(3.0, q, qn);
    const double b = __fma_rn(3.0, qn, q);
    return __fma_rn(p, a, -pmul(pn, b));
}

// (f1 - f0)(f1 + f0 + 4 c): the direction along a momentum component, from its
// values one point either side (f1, f0) and at the point (c).
__device__ __forceinline__ double along_term(double f1, double f0, double c) {
    return pmul(f1 - f0, __fma_rn(4.0, c, f1 + f0));
}

// One tile: columns [tile_x*32, +32) x [tile_y*TY, +TY) of the interior, levels
// [k0, k1), for one output mode (ADVANCE: forward Euler, else the tendency).
// Called by every thread of a (32, TY+1) block; `smem` holds
// FastSmem<TY>::doubles. Starts and ends with the exchange buffers free.
template <int NS, int MASK, int TY, bool ADVANCE>
__device__ __forceinline__ void fast_tile_mode(const AdvArgs &a, int tile_x, int tile_y, int k0, int k1,
                                               double *smem) {
    constexpr bool DU = MASK & 1, DV = (MASK >> 1) & 1, DW = (MASK >> 2) & 1, DS = NS > 0;
    constexpr bool filled = (MASK & kFillMask) != 0;  // F2C_ADVANCE_FILLED: outputs with their ghost images
    // face sums each point computes (at its north/east/top faces)
    constexpr bool F_UY = DU || DV, F_VX = DU || DV, F_UZ = DU || DW, F_WX = DU || DW, F_VZ = DV || DW,
                   F_WY = DV || DW;
    using Sm = FastSmem<TY>;
    const int lane = threadIdx.x;
    const int warp = threadIdx.y;
    const bool edge = warp == TY;
    const int i0 = tile_x * kFastTX, j0 = tile_y * TY;
    const int i = i0 + lane, j = j0 + warp;
    const bool active = !edge && i < a.nx && j < a.ny;
    const bool south_lane = edge && i < a.nx;                      // (i, j0-1)
    const bool west_lane = edge && lane < TY && j0 + lane < a.ny;  // (i0-1, j0+lane)
    const long long sx = a.sx, plane = a.plane;
    const double *__restrict__ U = a.u;
    const double *__restrict__ V = a.v;
    const double *__restrict__ W = a.w;
    const FastCoefficients c = a.f;
    const int cj = edge ? j0 - 1 : j;
    long long p = (long long)(i + a.h) + sx * (long long)(cj + a.h) + plane * (long long)(k0 + a.h);
    long long pw = (long long)(i0 - 1 + a.h) + sx * (long long)(j0 + lane + a.h) + plane * (long long)(k0 + a.h);
#define LD(A, q, di, dj, dk) __ldg((A) + (q) + (di) + (dj)*sx + (dk)*plane)

    // values of the level below, carried up the march: face sums at the top faces of level k-1, W there,
    // the vertical scaled velocity there, and this level's U, V, W (loaded as the level above).
    double bUz = 0, bWx = 0, bVz = 0, bWy = 0, bcW = 0, Wm = 0, U0 = 0, V0 = 0, W0 = 0;
    if (active) {
        const double Um = LD(U, p, 0, 0, -1), Vm = LD(V, p, 0, 0, -1);
        Wm = LD(W, p, 0, 0, -1);
        U0 = LD(U, p, 0, 0, 0);
        V0 = LD(V, p, 0, 0, 0);
        W0 = LD(W, p, 0, 0, 0);
        if (F_UZ) bUz = U0 + Um;
        if (F_WX) bWx = LD(W, p, 1, 0, -1) + Wm;
        if (F_VZ) bVz = V0 + Vm;
        if (F_WY) bWy = LD(W, p, 0, 1, -1) + Wm;
        if (DS) bcW = c.sz * Wm;
    }

    int buf = 0;
    for (int k = k0; k < k1; ++k, p += plane, pw += plane, buf ^= 1) {
        double *south = smem + buf * Sm::PER_BUFFER;  // [slot][TY+1][32]
        double *west = south + Sm::SOUTH;             // [slot][TY]
        constexpr int ROW = kFastTX, SLOT = (TY + 1) * kFastTX;
        // ---------------- own faces, handed to the neighbours ----------------
        double Up = 0, Vp = 0, Wp = 0;
        double sUy = 0, sVx = 0, sUz = 0, sWx = 0, sVz = 0, sWy = 0, cU = 0, cV = 0, cW = 0;
        if (active) {
            Up = LD(U, p, 0, 0, 1);
            Vp = LD(V, p, 0, 0, 1);
            Wp = LD(W, p, 0, 0, 1);
            if (F_UY) sUy = LD(U, p, 0, 1, 0) + U0;
            if (F_VX) sVx = LD(V, p, 1, 0, 0) + V0;
            if (F_UZ) sUz = Up + U0;
            if (F_WX) sWx = LD(W, p, 1, 0, 0) + W0;
            if (F_VZ) sVz = Vp + V0;
            if (F_WY) sWy = LD(W, p, 0, 1, 0) + W0;
            if (DS) {
                cU = pmul(c.sx, U0);
                cV = pmul(c.sy, V0);
                cW = pmul(c.sz, W0);
            }
            const int at = (warp + 1) * ROW + lane;
            if (DU) {
                south[0 * SLOT + at] = sUy;
                south[1 * SLOT + at] = sVx;
            }
            if (DW) {
                south[2 * SLOT + at] = sWy;
                south[3 * SLOT + at] = sVz;
            }
            if (DS) south[4 * SLOT + at] = cV;
        } else if (edge) {
            if (south_lane) {
                // north faces of row j0-1: the tile's south faces
                if (DU || DW) {
                    const double u0 = LD(U, p, 0, 0, 0), v0 = LD(V, p, 0, 0, 0);
                    if (DU) {
                        south[0 * SLOT + lane] = LD(U, p, 0, 1, 0) + u0;
                        south[1 * SLOT + lane] = LD(V, p, 1, 0, 0) + v0;
                    }
                    if (DW) {
                        south[2 * SLOT + lane] = LD(W, p, 0, 1, 0) + LD(W, p, 0, 0, 0);
                        south[3 * SLOT + lane] = LD(V, p, 0, 0, 1) + v0;
                    }
                    if (DS) south[4 * SLOT + lane] = c.sy * v0;
                } else if (DS) {
                    south[4 * SLOT + lane] = c.sy * LD(V, p, 0, 0, 0);
                }
            }
            if (west_lane) {
                // east faces of column i0-1 (row j0+lane): the tile's west faces
                if (DV || DW) {
                    const double u0 = LD(U, pw, 0, 0, 0);
                    if (DV) {
                        west[0 * TY + lane] = LD(V, pw, 1, 0, 0) + LD(V, pw, 0, 0, 0);
                        west[1 * TY + lane] = LD(U, pw, 0, 1, 0) + u0;
                    }
                    if (DW) {
                        west[2 * TY + lane] = LD(W, pw, 1, 0, 0) + LD(W, pw, 0, 0, 0);
                        west[3 * TY + lane] = LD(U, pw, 0, 0, 1) + u0;
                    }
                    if (DS) west[4 * TY + lane] = c.sx * u0;
                } else if (DS) {
                    west[4 * TY + lane] = c.sx * LD(U, pw, 0, 0, 0);
                }
            }
        }
        // x neighbours by shuffle (every lane of a compute warp takes part; lane 0 reads the west column below)
        double wVx = 0, wUy = 0, wWx = 0, wUz = 0, wcU = 0;
        if (!edge) {
            if (DV) {
                wVx = __shfl_up_sync(0xffffffffu, sVx, 1);
                wUy = __shfl_up_sync(0xffffffffu, sUy, 1);
            }
            if (DW) {
                wWx = __shfl_up_sync(0xffffffffu, sWx, 1);
                wUz = __shfl_up_sync(0xffffffffu, sUz, 1);
            }
            if (DS) wcU = __shfl_up_sync(0xffffffffu, cU, 1);
        }
        __syncthreads();
        // ---------------- the tendencies ----------------
        if (active) {
            if (lane == 0) {
                if (DV) {
                    wVx = west[0 * TY + warp];
                    wUy = west[1 * TY + warp];
                }
                if (DW) {
                    wWx = west[2 * TY + warp];
                    wUz = west[3 * TY + warp];
                }
                if (DS) wcU = west[4 * TY + warp];
            }
            const int at = warp * ROW + lane;  // the row south of this one
            if (DU) {
                const double X = along_term(LD(U, p, 1, 0, 0), LD(U, p, -1, 0, 0), U0);
                const double Y = cross_term(sUy, south[0 * SLOT + at], sVx, south[1 * SLOT + at]);
                const double Z = cross_term(sUz, bUz, sWx, bWx);
                double t = ADVANCE ? __fma_rn(c.cz, Z, U0) : pmul(c.cz, Z);
                t = __fma_rn(c.cy, Y, t);
                t = __fma_rn(c.gx, X, t);
                if (a.out[0]) { if (filled) store_filled(a.out[0], 0, a, i, j, k, t); else a.out[0][p] = t; }
            }
            if (DV) {
                const double X = cross_term(sVx, wVx, sUy, wUy);
                const double Y = along_term(LD(V, p, 0, 1, 0), LD(V, p, 0, -1, 0), V0);
                const double Z = cross_term(sVz, bVz, sWy, bWy);
                double t = ADVANCE ? __fma_rn(c.cz, Z, V0) : pmul(c.cz, Z);
                t = __fma_rn(c.gy, Y, t);
                t = __fma_rn(c.cx, X, t);
                if (a.out[1]) { if (filled) store_filled(a.out[1], 0, a, i, j, k, t); else a.out[1][p] = t; }
            }
            if (DW) {
                const double X = cross_term(sWx, wWx, sUz, wUz);
                const double Y = cross_term(sWy, south[2 * SLOT + at], sVz, south[3 * SLOT + at]);
                const double Z = along_term(Wp, Wm, W0);
                double t = ADVANCE ? __fma_rn(c.gz, Z, W0) : pmul(c.gz, Z);
                t = __fma_rn(c.cy, Y, t);
                t = __fma_rn(c.cx, X, t);
                if (a.out[2]) { if (filled) store_filled(a.out[2], 1, a, i, j, k, t); else a.out[2][p] = t; }
            }
            if (DS) {
                const double scV = south[4 * SLOT + at];
                const double D = ((wcU - cU) + (scV - cV)) + (bcW - cW);
#pragma unroll
                for (int n = 0; n < NS; ++n) {
                    const double *__restrict__ S = a.s[n];
                    const double S0 = LD(S, p, 0, 0, 0);
                    double t = ADVANCE ? __fma_rn(S0, D, S0) : pmul(S0, D);
                    t = __fma_rn(-cU, LD(S, p, 1, 0, 0), t);
                    t = __fma_rn(wcU, LD(S, p, -1, 0, 0), t);
                    t = __fma_rn(-cV, LD(S, p, 0, 1, 0), t);
                    t = __fma_rn(scV, LD(S, p, 0, -1, 0), t);
                    t = __fma_rn(-cW, LD(S, p, 0, 0, 1), t);
                    t = __fma_rn(bcW, LD(S, p, 0, 0, -1), t);
                    if (a.st[n]) { if (filled) store_filled(a.st[n], 0, a, i, j, k, t); else a.st[n][p] = t; }
                }
            }
            // carry up the march
            bUz = sUz; bWx = sWx; bVz = sVz; bWy = sWy; bcW = cW;
            Wm = W0;
            U0 = Up; V0 = Vp; W0 = Wp;
        }
    }
#undef LD
}

// The tile in the instance's output mode. The mode is a template argument of
// the tile so that a tendency's first term of each sum is a plain product
// (pmul, off the FP64 pipe) rather than an FMA with a zero addend, which a
// runtime choice would leave on the FP64 pipe; a filled advance is an advance.
template <int NS, int MASK, int TY>
__device__ __forceinline__ void fast_tile(const AdvArgs &a, int tile_x, int tile_y, int k0, int k1, double *smem) {
    if constexpr ((MASK & kFillMask) != 0) {
        fast_tile_mode<NS, MASK, TY, true>(a, tile_x, tile_y, k0, k1, smem);
    } else if (a.mode != 0) {
        fast_tile_mode<NS, MASK, TY, true>(a, tile_x, tile_y, k0, k1, smem);
    } else {
        fast_tile_mode<NS, MASK, TY, false>(a, tile_x, tile_y, k0, k1, smem);
    }
}

template <int NS, int MASK, int TY, int CTAS = fast_ctas_per_sm<TY>()>
__global__ void __launch_bounds__(fast_threads<TY>(), CTAS) advection_fast_kernel(const AdvArgs a) {
    __shared__ double smem[FastSmem<TY>::doubles];
    const int k0 = blockIdx.z * a.kz;
    fast_tile<NS, MASK, TY>(a, blockIdx.x, blockIdx.y, k0, min(k0 + a.kz, a.nz), smem);
}

// z-chunk depth of one launch: deep for large grids, shallower for small ones
// so that at least four CTAs per SM are available (down to two levels).
inline int fast_chunk_depth(int nx, int ny, int nz, int ty, int sms) {
    const long long tiles = (long long)((nx + kFastTX - 1) / kFastTX) * ((ny + ty - 1) / ty);
    const long long want = 4LL * (sms > 0 ? sms : 152);
    long long kz = (tiles * nz + want - 1) / want;
    if (kz > kFastKZ) kz = kFastKZ;
    if (kz < 2) kz = 2;
    return (int)kz;
}

template <int NS, int MASK, int TY>
cudaError_t launch_fast(const AdvArgs &a, int sms, cudaStream_t stream) {
    AdvArgs b = a;
    if (b.kz <= 0) b.kz = fast_chunk_depth(b.nx, b.ny, b.nz, TY, sms);
    const dim3 block(kFastTX, TY + 1, 1);
    const dim3 grid((b.nx + kFastTX - 1) / kFastTX, (b.ny + TY - 1) / TY, (b.nz + b.kz - 1) / b.kz);
    const long long ctas = (long long)grid.x * grid.y * grid.z;
    if (TY == kFastTY && ctas >= (long long)kFastDeepCtas * (sms > 0 ? sms : 152))
        advection_fast_kernel<NS, MASK, TY, kFastDeepCtasPerSM><<<grid, block, 0, stream>>>(b);
    else
        advection_fast_kernel<NS, MASK, TY><<<grid, block, 0, stream>>>(b);
    return cudaGetLastError();
}

} // namespace f2c
