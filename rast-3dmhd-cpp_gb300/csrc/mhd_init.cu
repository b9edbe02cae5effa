// mhd_init.cu -- initial state generated on the device.
//
// The reference builds its initial state on the host (Static(),
// 3dmhdphsic.h:549-763: a hydrostatic background from an ODE integration,
// RAN2 noise scattered from rank 0, an optional field layer).  A server that
// admits many simulations per second should not spend host time on that, so
// this kernel writes the synthetic polytropic state straight into HBM:
//   T = 1 + THETA z,  rho = T^m with m = GRAV/THETA - 1,
//   T *= 1 + noise * N(0, 1) on interior cells,
//   Bz = bz0 on interior planes (0 on the walls, where iBCon = 0 pins it),
//   zero momenta (with lShr: rho v = +rho / -rho on the top / bottom walls),
// with x/y ghosts as periodic images.  N(0, 1) is Box-Muller on two uniforms
// from splitmix64 (Steele, Lea and Flood 2014) of (seed, global interior
// cell index), so the field does not depend on the launch shape; the host
// mirror of this generator is mhd_gb300.case.device_initial_state.
#include "mhd_context.h"

#include <cmath>
#include <vector>

namespace {

__device__ __forceinline__ unsigned long long splitmix64(unsigned long long x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

// uniform in (0, 1]: 53 random bits
__device__ __forceinline__ double u01(unsigned long long h) { return ((h >> 11) + 1) * (1.0 / 9007199254740992.0); }

__global__ void k_init(Grid g, Fields8 U, const double* zc, double theta, double m, double noise,
                       unsigned long long seed, double bz0, int mag, int shr) {
    const long long n = (long long)g.nx * g.ny * g.nz;
    const int nPx = g.nx - 2, nPy = g.ny - 2;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(i % g.nx);
        const int y = (int)((i / g.nx) % g.ny);
        const int z = (int)(i / g.sz);
        const int xs = (x == 0) ? g.nx - 2 : (x == g.nx - 1 ? 1 : x);  // periodic image
        const int ys = (y == 0) ? g.ny - 2 : (y == g.ny - 1 ? 1 : y);
        const double t0 = 1.0 + theta * zc[z];
        const double ro = pow(t0, m);
        double tt = t0;
        if (z > 0 && z < g.nz - 1) {
            const unsigned long long cell =
                ((unsigned long long)(z - 1) * nPy + (unsigned long long)(ys - 1)) * nPx + (unsigned long long)(xs - 1);
            const unsigned long long h1 = splitmix64(seed ^ splitmix64(2 * cell));
            const unsigned long long h2 = splitmix64(seed ^ splitmix64(2 * cell + 1));
            const double r = sqrt(-2.0 * log(u01(h1)));
            const double gauss = r * cospi(2.0 * u01(h2));
            tt = t0 * (1.0 + noise * gauss);
        }
        U.p[S_TT][i] = tt;
        U.p[S_RO][i] = ro;
        U.p[S_RU][i] = 0.0;
        U.p[S_RW][i] = 0.0;
        double rv = 0.0;
        if (shr && z == 1) rv = ro;
        if (shr && z == g.nz - 2) rv = -ro;
        U.p[S_RV][i] = rv;
        if (mag) {
            U.p[S_BX][i] = 0.0;
            U.p[S_BY][i] = 0.0;
            U.p[S_BZ][i] = (z >= 2 && z <= g.nz - 3) ? bz0 : 0.0;
        }
    }
}

// horizontal mean of F over the interior of every z plane (one block per plane)
__global__ void k_plane_mean(Grid g, const double* F, double* out) {
    __shared__ double s[256];
    const int z = blockIdx.x, nx = g.nx - 2, n = nx * (g.ny - 2);
    double w = 0.0;
    for (int k = threadIdx.x; k < n; k += blockDim.x)
        w += F[(long long)z * g.sz + (long long)(1 + k / nx) * g.sy + 1 + k % nx];
    s[threadIdx.x] = w;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h) s[threadIdx.x] += s[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[z] = s[0] / ((double)nx * (g.ny - 2));
}

// FP32 storage: deviation of every FP64 field from its profile (rho0, T0 for RO, TT)
__global__ void k_to_f32(Grid g, int nf, Fields8 Z, Fields8f U, const double* rho0, const double* t0) {
    const long long n = (long long)g.nx * g.ny * g.nz;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int z = (int)(i / g.sz);
        for (int f = 0; f < nf; f++) {
            const double prof = (f == S_RO) ? rho0[z] : (f == S_TT) ? t0[z] : 0.0;
            U.p[f][i] = (float)(Z.p[f][i] - prof);
        }
    }
}

}  // namespace

extern "C" int mhd_init_polytrope(mhd_ctx* ctx, const double* zcoord, double noise, unsigned long long seed,
                                  double bz0) {
    if (!ctx || !zcoord) return MHD_ERR_INVALID;
    const int nz = ctx->g.nz;
    double* dz = nullptr;
    // the z coordinates (and, for FP32 contexts, the two plane-mean profiles)
    // go into the context's reduction scratch (it holds 8 x 1216 doubles)
    if ((size_t)3 * nz > (size_t)8 * ctx->red_blocks) return ctxops::fail(ctx, MHD_ERR_INVALID, "nz too large");
    dz = ctx->red;
    cudaError_t e = cudaMemcpyAsync(dz, zcoord, sizeof(double) * nz, cudaMemcpyHostToDevice, ctx->stream);
    if (e != cudaSuccess) return ctxops::fail(ctx, MHD_ERR_CUDA, cudaGetErrorString(e));
    const double theta = ctx->prm.THETA, m = ctx->prm.GRAV / ctx->prm.THETA - 1.0;
    const long long n = (long long)ctx->ncell;
    long long blocks = (n + 255) / 256;
    if (blocks > 152 * 32) blocks = 152 * 32;
    // FP32 contexts: the FP64 state goes into the RK register Z (which carries
    // the state between their steps), then into the FP32 deviation fields
    double* target = ctx->fp32 ? ctx->Zb : ctx->U[ctx->cur];
    k_init<<<(int)blocks, 256, 0, ctx->stream>>>(ctx->g, ctxops::fields_of(ctx, target), dz, theta, m,
                                                 noise, seed, bz0, (ctx->sw & kSwMag) ? 1 : 0,
                                                 (ctx->sw & kSwShr) ? 1 : 0);
    e = cudaGetLastError();
    if (e != cudaSuccess) return ctxops::fail(ctx, MHD_ERR_CUDA, cudaGetErrorString(e));
    if (ctx->fp32) {
        const Fields8 Z = ctxops::fields_of(ctx, ctx->Zb);
        double* means = ctx->red + nz;  // rho0, T0
        k_plane_mean<<<nz, 256, 0, ctx->stream>>>(ctx->g, Z.p[S_RO], means);
        k_plane_mean<<<nz, 256, 0, ctx->stream>>>(ctx->g, Z.p[S_TT], means + nz);
        e = cudaMemcpyAsync(ctx->h_bg.data(), means, sizeof(double) * 2 * nz, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) return ctxops::fail(ctx, MHD_ERR_CUDA, cudaGetErrorString(e));
        const int rc = ctxops::profiles_from_means(ctx);
        if (rc) return rc;
        k_to_f32<<<(int)blocks, 256, 0, ctx->stream>>>(ctx->g, ctx->nf, Z, ctxops::fields32_of(ctx, ctx->U32[ctx->cur]),
                                                      ctx->d_bg, ctx->d_bg + nz);
        e = cudaGetLastError();
        if (e != cudaSuccess) return ctxops::fail(ctx, MHD_ERR_CUDA, cudaGetErrorString(e));
    }
    ctx->ghosts_synced = false;
    e = cudaStreamSynchronize(ctx->stream);  // the host z array may go away after return
    return e == cudaSuccess ? MHD_OK : ctxops::fail(ctx, MHD_ERR_CUDA, cudaGetErrorString(e));
}
