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

}  // namespace

extern "C" int mhd_init_polytrope(mhd_ctx* ctx, const double* zcoord, double noise, unsigned long long seed,
                                  double bz0) {
    if (!ctx || !zcoord) return MHD_ERR_INVALID;
    if (ctx->fp32) return ctxops::fail(ctx, MHD_ERR_UNSUPPORTED, "device initialisation writes FP64 contexts");
    const int nz = ctx->g.nz;
    double* dz = nullptr;
    // the z coordinates go into the context's reduction scratch (nz doubles fit: it holds 8 x 1216)
    if ((size_t)nz > (size_t)8 * ctx->red_blocks) return ctxops::fail(ctx, MHD_ERR_INVALID, "nz too large");
    dz = ctx->red;
    cudaError_t e = cudaMemcpyAsync(dz, zcoord, sizeof(double) * nz, cudaMemcpyHostToDevice, ctx->stream);
    if (e != cudaSuccess) return ctxops::fail(ctx, MHD_ERR_CUDA, cudaGetErrorString(e));
    const double theta = ctx->prm.THETA, m = ctx->prm.GRAV / ctx->prm.THETA - 1.0;
    const long long n = (long long)ctx->ncell;
    long long blocks = (n + 255) / 256;
    if (blocks > 152 * 32) blocks = 152 * 32;
    k_init<<<(int)blocks, 256, 0, ctx->stream>>>(ctx->g, ctxops::fields_of(ctx, ctx->U[ctx->cur]), dz, theta, m,
                                                 noise, seed, bz0, (ctx->sw & kSwMag) ? 1 : 0,
                                                 (ctx->sw & kSwShr) ? 1 : 0);
    e = cudaGetLastError();
    if (e != cudaSuccess) return ctxops::fail(ctx, MHD_ERR_CUDA, cudaGetErrorString(e));
    ctx->ghosts_synced = false;
    e = cudaStreamSynchronize(ctx->stream);  // the host z array may go away after return
    return e == cudaSuccess ? MHD_OK : ctxops::fail(ctx, MHD_ERR_CUDA, cudaGetErrorString(e));
}
