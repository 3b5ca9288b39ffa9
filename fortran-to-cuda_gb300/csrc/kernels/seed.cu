// Seeded synthetic advection fields written on the device (include/f2c_serve.h).
//
// A server defines each admitted job's first field set where it will stay, in
// the job's device mirrors, instead of generating it on the host and moving it
// over NVLink-C2C. The recipe is the sine-mode one of the host workload
// generator (four modes per velocity at its staggered position, N(0, 0.05)
// noise on the interior, scalars uniform or Gaussian blobs); the random draws
// come from a counter-based generator (splitmix64 mixing of a per-field key
// and the point's interior index, normals by the Box-Muller transform), so
// every value depends on the seed and the geometry alone. The velocities and
// blobs are evaluated in single precision and stored as FP64.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <string>

#include "../../../include/f2c_serve.h"

namespace f2c {
int fail(int status, const std::string &message);
int check_grid(const f2c_grid_v1 *g);

namespace {

constexpr double kTwoPi = 6.283185307179586;

__host__ __device__ inline uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// A uniform double in [0, 1) from 53 bits of the n-th draw of stream `key`.
__host__ __device__ inline double uniform(uint64_t key, uint64_t n) {
    return (double)(mix64(key + 0x9E3779B97F4A7C15ull * (n + 1)) >> 11) * 0x1.0p-53;
}

// A uniform float in [0, 1) from the top 24 bits of the n-th draw of stream `key`.
__host__ __device__ inline float uniform24(uint64_t key, uint64_t n) {
    return (float)(mix64(key + 0x9E3779B97F4A7C15ull * (n + 1)) >> 40) * 0x1.0p-24f;
}

struct Mode {
    float ax, ay, az, phi;  // 2 pi k / L per axis, phase
};

struct SeedArgs {
    double *f[3 + F2C_MAX_SCALARS];
    Mode mode[3][4];
    uint64_t key[3 + F2C_MAX_SCALARS];
    int nscalar;
    int nx, ny, nz, h;
    long long sx, plane;
    float dx, dy, dz;
    float blob_cz[F2C_MAX_SCALARS];  // blob centres along z (fraction of Lz)
};

// The modes, the noise and the blobs are evaluated in single precision (the
// values are synthetic inputs; FP64 sin, log and exp would cost GB300's FP64
// pipe several advection steps' worth of work per job) and stored as FP64;
// the uniform scalars keep 53 random bits.
__global__ void __launch_bounds__(256) seed_kernel(SeedArgs a) {
    const long long points = (long long)a.nx * a.ny * a.nz;
    const float lx = a.nx * a.dx, ly = a.ny * a.dy, lz = a.nz * a.dz;
    const float sigma = 0.125f * fminf(lx, fminf(ly, lz));
    for (long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x; n < points;
         n += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(n % a.nx);
        const int j = (int)((n / a.nx) % a.ny);
        const int k = (int)(n / ((long long)a.nx * a.ny));
        const long long at = (long long)(i + a.h) + a.sx * (j + a.h) + a.plane * (k + a.h);
        for (int c = 0; c < 3; ++c) {
            // staggered position: U on east faces, V on north faces, W on top faces
            const float x = (i + (c == 0 ? 1.0f : 0.5f)) * a.dx;
            const float y = (j + (c == 1 ? 1.0f : 0.5f)) * a.dy;
            const float z = (k + (c == 2 ? 1.0f : 0.5f)) * a.dz;
            float v = 0.0f;
            for (int m = 0; m < 4; ++m) {
                const Mode &q = a.mode[c][m];
                v += sinf(q.az * z + q.ay * y + (q.ax * x + q.phi));
            }
            const float u1 = 1.0f - uniform24(a.key[c], 2 * (uint64_t)n);  // (0, 1]
            const float u2 = uniform24(a.key[c], 2 * (uint64_t)n + 1);
            v += 0.05f * (sqrtf(-2.0f * logf(u1)) * cosf(6.28318530717958648f * u2));
            a.f[c][at] = (double)v;
        }
        for (int s = 0; s < a.nscalar; ++s) {
            double v;
            if (s == 0) {
                v = 280.0 + 20.0 * uniform(a.key[3], (uint64_t)n);
            } else if (s == 1) {
                v = 0.02 * uniform(a.key[4], (uint64_t)n);
            } else {
                const float x = (i + 0.5f) * a.dx - 0.5f * lx, y = (j + 0.5f) * a.dy - 0.5f * ly,
                            z = (k + 0.5f) * a.dz - a.blob_cz[s] * lz;
                v = (double)expf(-(x * x + y * y + z * z) / (2.0f * sigma * sigma));
            }
            a.f[3 + s][at] = v;
        }
    }
}

}  // namespace
}  // namespace f2c

using namespace f2c;

extern "C" int f2c_seed_fields_v1(const f2c_grid_v1 *grid, uint64_t seed, int32_t nscalar, double *const *fields,
                                  void *stream) {
    if (int s = check_grid(grid)) return s;
    if (nscalar < 0 || nscalar > F2C_MAX_SCALARS) return fail(1, "scalar count out of range");
    if (!fields) return fail(1, "null field list");
    if (grid->nz < grid->halo || grid->nx < grid->halo || grid->ny < grid->halo)
        return fail(1, "seeded fields need nx, ny, nz >= halo (for the boundary fill)");
    SeedArgs a{};
    const int count = 3 + nscalar;
    for (int c = 0; c < count; ++c) {
        if (!fields[c]) return fail(1, "null field pointer");
        a.f[c] = fields[c];
    }
    a.nscalar = nscalar;
    a.nx = (int)grid->nx; a.ny = (int)grid->ny; a.nz = (int)grid->nz; a.h = (int)grid->halo;
    a.sx = grid->sx;
    a.plane = grid->sx * grid->sy;
    a.dx = (float)grid->dx; a.dy = (float)grid->dy; a.dz = (float)grid->dz;
    // the host draws the modes: per velocity and mode kx, ky, kz in 1..4, then the phase
    uint64_t state = mix64(seed ^ 0x5EEDF1E1D5ull);
    auto next = [&] { state += 0x9E3779B97F4A7C15ull; return mix64(state); };
    const double len[3] = {a.nx * grid->dx, a.ny * grid->dy, a.nz * grid->dz};
    for (int c = 0; c < 3; ++c)
        for (int m = 0; m < 4; ++m) {
            const double kx = 1.0 + (double)(next() % 4), ky = 1.0 + (double)(next() % 4), kz = 1.0 + (double)(next() % 4);
            a.mode[c][m] = {(float)(kTwoPi * kx / len[0]), (float)(kTwoPi * ky / len[1]), (float)(kTwoPi * kz / len[2]),
                            (float)(kTwoPi * ((double)(next() >> 11) * 0x1.0p-53))};
        }
    for (int c = 0; c < 3 + F2C_MAX_SCALARS; ++c) a.key[c] = next();
    for (int s = 0; s < F2C_MAX_SCALARS; ++s) a.blob_cz[s] = 0.25f + 0.25f * (s - 2);
    const cudaStream_t s = static_cast<cudaStream_t>(stream);
    const long long points = (long long)a.nx * a.ny * a.nz;
    int sms = 0, device = 0;
    if (cudaGetDevice(&device) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
        sms = 152;
    const long long blocks = std::min<long long>((points + 255) / 256, (long long)sms * 8);
    seed_kernel<<<(unsigned)blocks, 256, 0, s>>>(a);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(6, std::string("seed launch: ") + cudaGetErrorString(e));
    int32_t kinds[3 + F2C_MAX_SCALARS];
    for (int c = 0; c < count; ++c) kinds[c] = c == 2 ? 1 : 0;
    return f2c_halo_fill_v1(grid, fields, kinds, count, stream);
}
