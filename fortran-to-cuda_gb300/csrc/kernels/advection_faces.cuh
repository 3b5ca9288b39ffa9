// Face-sharing z-marching advection kernel for sm_103a.
//
// GB300 executes FP64 arithmetic at about 1.6 lane-operations per clock per SM
// (measured), some 75x below its FP32 rate, so this FP64 stencil is bound by
// the FP64 pipe long before HBM. The kernel therefore performs every distinct
// operation of the reference's per-point expression trees exactly once per
// grid point:
//
//  * Each flux on a cell face appears in the expressions of the two points
//    that share the face, with the same operands in the same order (IEEE
//    addition and multiplication commute exactly), so it is computed once:
//    top faces are carried in registers up the z-march, east and north faces
//    go through shared memory to the neighbour, and a ninth "edge" warp
//    supplies the tile's west column and south row.
//  * Sums shared between the CDU, CDV and CDW trees (e.g. U(j+1)+U feeds the
//    CDU y-flux, the CDV x-flux and the CDV advective average) are computed
//    once.
//  * The final multiplication by 0.5 (benchmarks/cdu/src/cdu.f90:39) is an
//    exact exponent decrement, done on the integer pipe (with the correctly
//    rounded subnormal case handled in integer arithmetic as well).
//
// Every other operation follows the reference grouping (advection_point.cuh),
// so results are bit-identical to the oracle. The advective-form products and
// the second product of each face flux are computed on the integer pipes (pmul
// below, rounded exactly as DMUL): 27 of the 48 products per point with three
// scalars. That split balances the pipes; measured at 512 x 512 x 128 with
// three scalars (two CTAs per SM): 8.74 ms with every product a DMUL, 8.17 ms with all 48 on the
// integer pipes (the FP64 pipe then waits on the longer integer chains, 62 %
// busy), 7.33 ms with these 27 (7.69 with the advective ones alone, 7.46 with
// both flux products as well). Operation count per point:
// U, V, W: 9 face sums + 18 flux products + 15 flux differences + 48
// advective-form operations = 90; scalars: 3 shared coefficient products +
// 11 per scalar.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "advection_kernels.cuh"
#include "device.cuh"
#include "soft_fp64.cuh"

namespace f2c {

// Products on the integer pipes (soft_fp64.cuh): bit-identical to DMUL, they
// take multiplications off the FP64 pipe that bounds these kernels. Additions
// stay on the FP64 pipe: an integer addition costs about as much time on the
// ALU pipe as it saves on the FP64 one (measured slower).
__device__ __forceinline__ double pmul(double a, double b) { return mul_rn_int(a, b); }

constexpr int kFaceTX = 32;       // points per tile along x (one warp)
constexpr int kFaceTY = 8;        // compute warps per tile (points along y)
constexpr int kFaceKZ = 32;       // levels per z-chunk
constexpr int kFaceThreads = kFaceTX * (kFaceTY + 1);
// Three CTAs per SM (72 registers a thread, a few spills served by L1): 27
// warps hide the FP64, integer and shared-memory latencies. What made room for
// the third CTA is phase B reading the point's own fluxes back from the shared
// rows and its values again from L1 (ldg_again) instead of holding them in
// registers across the barrier. Measured at 512 x 512 x 128 with three
// scalars: 7.33 ms at two CTAs before that change (8.04 at three, with twice
// the spills), 7.26 ms at two and 7.11 at three after it.
constexpr int kFaceCtasPerSM = 3;

// Exact x * 0.5 without the FP64 pipe: for normal x the exponent field drops by
// one; for the smallest normals and subnormals the significand shifts right
// with round-half-even, which is what the correctly rounded product does.
// Infinities and NaNs are returned unchanged.
__device__ __forceinline__ double exact_half(double x) {
    const long long b = __double_as_longlong(x);
    const unsigned e = (unsigned)((unsigned long long)b >> 52) & 0x7ffu;
    const long long sign = b & (long long)0x8000000000000000ULL;
    const long long m = b & 0x001fffffffffffffLL;  // significand (with the lowest exponent bit for e == 1)
    const long long small = sign | ((m >> 1) + (m & (m >> 1) & 1));
    long long r = b - (1LL << 52);
    r = e < 2 ? small : r;
    r = e == 0x7ffu ? b : r;
    return __longlong_as_double(r);
}

// IEEE negation (the sign bit flipped, exact for every value) on the integer
// pipe. Written as inline PTX so that it stays an integer operation: a plain
// `-x`, or a sign flip written in C++, becomes a floating negation that the
// compiler issues on the FP64 pipe here (measured: three FP64 additions per
// point fewer, 2 % faster, results unchanged).
__device__ __forceinline__ double opaque_negate(double x) {
    unsigned long long r;
    asm("xor.b64 %0, %1, 0x8000000000000000;" : "=l"(r) : "l"((unsigned long long)__double_as_longlong(x)));
    return __longlong_as_double((long long)r);
}

// A read-only global load the compiler must issue where it stands (not merged
// with an earlier load of the same address), so that a value loaded before the
// tile's barrier need not stay in a register across it.
__device__ __forceinline__ double ldg_again(const double *q) {
    double v;
    asm volatile("ld.global.nc.f64 %0, [%1];" : "=d"(v) : "l"(q));
    return v;
}

template <int NS, int MASK>
struct FaceSmem {
    static constexpr int NF = 3 + NS;
    // [buffer][flux][row][column]: x faces have TX+1 columns (column 0 = west edge),
    // y faces TY+1 rows (row 0 = south edge).
    static constexpr int XF = kFaceTY * (kFaceTX + 1);
    static constexpr int YF = (kFaceTY + 1) * kFaceTX;
    static constexpr size_t bytes = sizeof(double) * 2 * NF * (XF + YF);
};

// One tile: columns [tx*32, tx*32+32) x [ty*8, ty*8+8) of the interior, levels
// [k0, k1). Called by every thread of a (32, 9) block; `smem` holds
// FaceSmem<NS, MASK>::bytes. Starts and ends with the shared face buffers free.
template <int NS, int MASK>
__device__ __forceinline__ void faces_tile(const AdvArgs &a, int tile_x, int tile_y, int k0, int k1, double *smem) {
    constexpr bool DO_U = MASK & 1, DO_V = MASK & 2, DO_W = MASK & 4, FILL = (MASK & kFillMask) != 0;
    using Smem = FaceSmem<NS, MASK>;
    constexpr int NF = Smem::NF;
    double *xface = smem;                         // [2][NF][XF]
    double *yface = smem + 2 * NF * Smem::XF;     // [2][NF][YF]

    const int lane = threadIdx.x;
    const int warp = threadIdx.y;
    const bool edge = warp == kFaceTY;
    const int i0 = tile_x * kFaceTX, j0 = tile_y * kFaceTY;
    const long long sx = a.sx, plane = a.plane;
    const double *__restrict__ U = a.u;
    const double *__restrict__ V = a.v;
    const double *__restrict__ W = a.w;
    const Coefficients c = a.c;

    // Compute threads own (i, j); the edge warp's lanes own (i0+lane, j0-1) for the south row and
    // (i0-1, j0+lane) for the west column.
    const int i = i0 + lane, j = j0 + warp;
    const bool active = !edge && i < a.nx && j < a.ny;
    const bool south_lane = edge && i < a.nx;
    const bool west_lane = edge && lane < kFaceTY && j0 + lane < a.ny;
    const int ci = edge ? i : i, cj = edge ? j0 - 1 : j;  // column of the south-row role
    long long p = (long long)(ci + a.h) + sx * (long long)(cj + a.h) + plane * (long long)(k0 + a.h);
    long long pw = (long long)(i0 - 1 + a.h) + sx * (long long)(j0 + lane + a.h) + plane * (long long)(k0 + a.h);
#define LD(A, q, di, dj, dk) __ldg((A) + (q) + (di) + (dj)*sx + (dk)*plane)

    // Top-face fluxes of the level below the current one (bottom faces), carried up the march.
    double FUzb = 0.0, FVzb = 0.0, FWzb = 0.0, ftb[NS > 0 ? NS : 1];
    if (active) {
        // prologue: top faces of level k0-1
        const double Um = LD(U, p, 0, 0, -1), U0 = LD(U, p, 0, 0, 0);
        const double Vm = LD(V, p, 0, 0, -1), V0 = LD(V, p, 0, 0, 0);
        const double Wm = LD(W, p, 0, 0, -1), W0 = LD(W, p, 0, 0, 0);
        if (DO_U) {
            const double sUz = U0 + Um;
            const double sWx = LD(W, p, 1, 0, -1) + Wm;
            FUzb = (c.Az * sUz) * sWx;
        }
        if (DO_V || DO_W) {
            const double sVz = V0 + Vm;
            const double sWy = LD(W, p, 0, 1, -1) + Wm;
            if (DO_V) FVzb = (c.Az * sVz) * sWy;
        }
        if (DO_W) {
            const double sWz = W0 + Wm;
            FWzb = (c.Az * sWz) * sWz;
        }
#pragma unroll
        for (int n = 0; n < NS; ++n) {
            const double *__restrict__ S = a.s[n];
            ftb[n] = (c.Sz * Wm) * (LD(S, p, 0, 0, 0) + LD(S, p, 0, 0, -1));
        }
    }

    int buf = 0;
    for (int k = k0; k < k1; ++k, p += plane, pw += plane, buf ^= 1) {
        double *xf = xface + buf * NF * Smem::XF;
        double *yf = yface + buf * NF * Smem::YF;
        // ---------------- phase A: own east / north / top faces, edge faces ----------------
        double U0 = 0, Ue = 0, Un = 0, Up = 0, V0 = 0, Ve = 0, Vn = 0, Vp = 0, W0 = 0, We = 0, Wn = 0, Wp = 0;
        double sUx = 0, sVx = 0, sWx = 0, sUy = 0, sVy = 0, sWy = 0, sUz = 0, sVz = 0, sWz = 0;
        double FUx = 0, FVx = 0, FWx = 0, FUy = 0, FVy = 0, FWy = 0, FUz = 0, FVz = 0, FWz = 0;
        double S0[NS > 0 ? NS : 1], fe[NS > 0 ? NS : 1], fn[NS > 0 ? NS : 1], ft[NS > 0 ? NS : 1];
        if (active) {
            U0 = LD(U, p, 0, 0, 0); Ue = LD(U, p, 1, 0, 0); Un = LD(U, p, 0, 1, 0); Up = LD(U, p, 0, 0, 1);
            V0 = LD(V, p, 0, 0, 0); Ve = LD(V, p, 1, 0, 0); Vn = LD(V, p, 0, 1, 0); Vp = LD(V, p, 0, 0, 1);
            W0 = LD(W, p, 0, 0, 0); We = LD(W, p, 1, 0, 0); Wn = LD(W, p, 0, 1, 0); Wp = LD(W, p, 0, 0, 1);
            if (DO_U) sUx = Ue + U0;
            if (DO_U || DO_V) sVx = Ve + V0;
            if (DO_U || DO_W) sWx = We + W0;
            if (DO_U || DO_V) sUy = Un + U0;
            if (DO_V) sVy = Vn + V0;
            if (DO_V || DO_W) sWy = Wn + W0;
            if (DO_U || DO_W) sUz = Up + U0;
            if (DO_V || DO_W) sVz = Vp + V0;
            if (DO_W) sWz = Wp + W0;
            if (DO_U) {
                FUx = pmul(c.Ax * sUx, sUx);
                FUy = pmul(c.Ay * sUy, sVx);
                FUz = pmul(c.Az * sUz, sWx);
            }
            if (DO_V) {
                FVx = pmul(c.Ax * sVx, sUy);
                FVy = pmul(c.Ay * sVy, sVy);
                FVz = pmul(c.Az * sVz, sWy);
            }
            if (DO_W) {
                FWx = pmul(c.Ax * sWx, sUz);
                FWy = pmul(c.Ay * sWy, sVz);
                FWz = pmul(c.Az * sWz, sWz);
            }
            if (NS > 0) {
                const double SxU = c.Sx * U0, SyV = c.Sy * V0, SzW = c.Sz * W0;
#pragma unroll
                for (int n = 0; n < NS; ++n) {
                    const double *__restrict__ S = a.s[n];
                    S0[n] = LD(S, p, 0, 0, 0);
                    fe[n] = SxU * (LD(S, p, 1, 0, 0) + S0[n]);
                    fn[n] = SyV * (LD(S, p, 0, 1, 0) + S0[n]);
                    ft[n] = SzW * (LD(S, p, 0, 0, 1) + S0[n]);
                }
            }
            const int xo = warp * (kFaceTX + 1) + lane + 1;
            const int yo = (warp + 1) * kFaceTX + lane;
            if (DO_U) { xf[0 * Smem::XF + xo] = FUx; yf[0 * Smem::YF + yo] = FUy; }
            if (DO_V) { xf[1 * Smem::XF + xo] = FVx; yf[1 * Smem::YF + yo] = FVy; }
            if (DO_W) { xf[2 * Smem::XF + xo] = FWx; yf[2 * Smem::YF + yo] = FWy; }
#pragma unroll
            for (int n = 0; n < NS; ++n) {
                xf[(3 + n) * Smem::XF + xo] = fe[n];
                yf[(3 + n) * Smem::YF + yo] = fn[n];
            }
        } else if (edge) {
            if (south_lane) {
                // north faces of row j0-1 (the tile's south faces)
                const double u0 = LD(U, p, 0, 0, 0), un = LD(U, p, 0, 1, 0);
                const double v0 = LD(V, p, 0, 0, 0), ve = LD(V, p, 1, 0, 0), vn = LD(V, p, 0, 1, 0);
                const double vp = LD(V, p, 0, 0, 1);
                const double w0 = LD(W, p, 0, 0, 0), wn = LD(W, p, 0, 1, 0);
                const int yo = lane;
                if (DO_U) {
                    const double s_uy = un + u0, s_vx = ve + v0;
                    yf[0 * Smem::YF + yo] = (c.Ay * s_uy) * s_vx;
                }
                if (DO_V) {
                    const double s_vy = vn + v0;
                    yf[1 * Smem::YF + yo] = (c.Ay * s_vy) * s_vy;
                }
                if (DO_W) {
                    const double s_wy = wn + w0, s_vz = vp + v0;
                    yf[2 * Smem::YF + yo] = (c.Ay * s_wy) * s_vz;
                }
                if (NS > 0) {
                    const double SyV = c.Sy * v0;
#pragma unroll
                    for (int n = 0; n < NS; ++n) {
                        const double *__restrict__ S = a.s[n];
                        yf[(3 + n) * Smem::YF + yo] = SyV * (LD(S, p, 0, 1, 0) + LD(S, p, 0, 0, 0));
                    }
                }
            }
            if (west_lane) {
                // east faces of column i0-1 (the tile's west faces), row j0+lane
                const double u0 = LD(U, pw, 0, 0, 0), ue = LD(U, pw, 1, 0, 0), un = LD(U, pw, 0, 1, 0);
                const double up = LD(U, pw, 0, 0, 1);
                const double v0 = LD(V, pw, 0, 0, 0), ve = LD(V, pw, 1, 0, 0);
                const double w0 = LD(W, pw, 0, 0, 0), we = LD(W, pw, 1, 0, 0);
                const int xo = lane * (kFaceTX + 1);
                if (DO_U) {
                    const double s_ux = ue + u0;
                    xf[0 * Smem::XF + xo] = (c.Ax * s_ux) * s_ux;
                }
                if (DO_V) {
                    const double s_vx = ve + v0, s_uy = un + u0;
                    xf[1 * Smem::XF + xo] = (c.Ax * s_vx) * s_uy;
                }
                if (DO_W) {
                    const double s_wx = we + w0, s_uz = up + u0;
                    xf[2 * Smem::XF + xo] = (c.Ax * s_wx) * s_uz;
                }
                if (NS > 0) {
                    const double SxU = c.Sx * u0;
#pragma unroll
                    for (int n = 0; n < NS; ++n) {
                        const double *__restrict__ S = a.s[n];
                        xf[(3 + n) * Smem::XF + xo] = SxU * (LD(S, pw, 1, 0, 0) + LD(S, pw, 0, 0, 0));
                    }
                }
            }
        }
        __syncthreads();
        // ---------------- phase B: differences of fluxes and the advective forms ----------------
        if (active) {
            const int xw = warp * (kFaceTX + 1) + lane;
            const int ys = warp * kFaceTX + lane;
            // this point's own east / north fluxes are read back from the shared rows and its values again
            // from memory (L1), rather than held in registers across the barrier
            const int xo = xw + 1, yo = ys + kFaceTX;
#define LDA(A, di, dj, dk) ldg_again((A) + p + (di) + (dj)*sx + (dk)*plane)
            const double Uc = LDA(U, 0, 0, 0), Vc = LDA(V, 0, 0, 0), Wc = LDA(W, 0, 0, 0);  // the point's own values
            const double Uw = LD(U, p, -1, 0, 0), Us = LD(U, p, 0, -1, 0), Um = LD(U, p, 0, 0, -1);
            const double Vw = LD(V, p, -1, 0, 0), Vs = LD(V, p, 0, -1, 0), Vm = LD(V, p, 0, 0, -1);
            const double Ww = LD(W, p, -1, 0, 0), Ws = LD(W, p, 0, -1, 0), Wm = LD(W, p, 0, 0, -1);
            if (DO_U) {
                const double r = opaque_negate(((xf[0 * Smem::XF + xo] - xf[0 * Smem::XF + xw]) + (yf[0 * Smem::YF + yo] - yf[0 * Smem::YF + ys])) + (FUz - FUzb));
                const double Vadv = (sVx + Vs) + LD(V, p, 1, -1, 0);
                const double Wadv = (sWx + Wm) + LD(W, p, 1, 0, -1);
                const double adv = (pmul(pmul(c.Bux, LDA(U, 1, 0, 0) - Uw), Uc) + pmul(pmul(c.Buy, LDA(U, 0, 1, 0) - Us), Vadv)) + pmul(pmul(c.Buz, LDA(U, 0, 0, 1) - Um), Wadv);
                if (a.out[0]) store_point_t<FILL>(a.out[0], U, p, exact_half(r - adv), a, 0, i, j, k);
                FUzb = FUz;
            }
            if (DO_V) {
                const double r = opaque_negate(((yf[1 * Smem::YF + yo] - yf[1 * Smem::YF + ys]) + (xf[1 * Smem::XF + xo] - xf[1 * Smem::XF + xw])) + (FVz - FVzb));
                const double Uadv = (sUy + Uw) + LD(U, p, -1, 1, 0);
                const double Wadv = (sWy + Wm) + LD(W, p, 0, 1, -1);
                const double adv = (pmul(pmul(c.Bvx, LDA(V, 1, 0, 0) - Vw), Uadv) + pmul(pmul(c.Bvy, LDA(V, 0, 1, 0) - Vs), Vc)) + pmul(pmul(c.Bvz, LDA(V, 0, 0, 1) - Vm), Wadv);
                if (a.out[1]) store_point_t<FILL>(a.out[1], V, p, exact_half(r - adv), a, 0, i, j, k);
                FVzb = FVz;
            }
            if (DO_W) {
                const double r = opaque_negate(((FWz - FWzb) + (yf[2 * Smem::YF + yo] - yf[2 * Smem::YF + ys])) + (xf[2 * Smem::XF + xo] - xf[2 * Smem::XF + xw]));
                const double Uadv = (sUz + Uw) + LD(U, p, -1, 0, 1);
                const double Vadv = (sVz + Vs) + LD(V, p, 0, -1, 1);
                const double adv = (pmul(pmul(c.Bwx, LDA(W, 1, 0, 0) - Ww), Uadv) + pmul(pmul(c.Bwy, LDA(W, 0, 1, 0) - Ws), Vadv)) + pmul(pmul(c.Bwz, LDA(W, 0, 0, 1) - Wm), Wc);
                if (a.out[2]) store_point_t<FILL>(a.out[2], W, p, exact_half(r - adv), a, 1, i, j, k);
                FWzb = FWz;
            }
#pragma unroll
            for (int n = 0; n < NS; ++n) {
                const double st = opaque_negate(((xf[(3 + n) * Smem::XF + xo] - xf[(3 + n) * Smem::XF + xw]) + (yf[(3 + n) * Smem::YF + yo] - yf[(3 + n) * Smem::YF + ys])) +
                                    (ft[n] - ftb[n]));
                if (a.st[n]) store_point_t<FILL>(a.st[n], a.s[n], p, st, a, 0, i, j, k);
                ftb[n] = ft[n];
            }
#undef LDA
        }
    }
#undef LD
}

template <int NS, int MASK>
__global__ void __launch_bounds__(kFaceThreads, kFaceCtasPerSM) advection_faces_kernel(const AdvArgs a) {
    extern __shared__ double smem[];
    const int k0 = blockIdx.z * a.kz;
    faces_tile<NS, MASK>(a, blockIdx.x, blockIdx.y, k0, min(k0 + a.kz, a.nz), smem);
}

// Depth of the z-chunks of one launch: deep (kFaceKZ) when the grid has work
// for several waves of CTAs, shallower for small grids so that at least four
// CTAs per SM are available (down to two levels, where the per-chunk prologue
// stays a small fraction of the work).
inline int chunk_depth(int nx, int ny, int nz) {
    const int sms = current_sm_count();
    const long long tiles = (long long)((nx + kFaceTX - 1) / kFaceTX) * ((ny + kFaceTY - 1) / kFaceTY);
    const long long want = 4LL * sms;
    long long kz = (tiles * nz + want - 1) / want;
    if (kz > kFaceKZ) kz = kFaceKZ;
    if (kz < 2) kz = 2;
    return (int)kz;
}

template <int NS, int MASK>
cudaError_t launch_faces(const AdvArgs &a, cudaStream_t stream) {
    using Smem = FaceSmem<NS, MASK>;
    static std::atomic<unsigned long long> configured{0};
    const cudaError_t e =
        configure_shared_once(configured, (const void *)advection_faces_kernel<NS, MASK>, (int)Smem::bytes);
    if (e != cudaSuccess) return e;
    AdvArgs b = a;
    if (b.kz <= 0) b.kz = chunk_depth(b.nx, b.ny, b.nz);
    const dim3 block(kFaceTX, kFaceTY + 1, 1);
    const dim3 grid((b.nx + kFaceTX - 1) / kFaceTX, (b.ny + kFaceTY - 1) / kFaceTY, (b.nz + b.kz - 1) / b.kz);
    advection_faces_kernel<NS, MASK><<<grid, block, Smem::bytes, stream>>>(b);
    return cudaGetLastError();
}

} // namespace f2c
