// mhd_diag.cu -- global diagnostics of the state: total mass, total energy,
// max |div B| and sanity flags.  The reference has no such diagnostics; they
// are reported for the FP32-storage runs and for failure detection.
//   mass   = sum rho dV
//   energy = sum (|rho u|^2 / (2 rho) + CV rho T + OBETA |B|^2 / 2) dV
//   divB   = max |D1x Bx + D1y By + D1z Bz| over interior, non-wall cells
// with dV = DDX[x] DDY[y] DDZ[z].  Per-block partials are folded by one block
// in a fixed order, so the result is deterministic.
#include "mhd_common.cuh"

namespace mhd {
namespace {

constexpr int kDiagThreads = 256;

template <bool MAG>
__global__ void k_diag(Grid g, Consts c, Fields8 U, double* part) {
    const int nPx = g.nx - 2, nPy = g.ny - 2, nPz = g.nz - 2;
    const long long ncell = (long long)nPx * nPy * nPz;
    double mass = 0, energy = 0, divb = 0, flags = 0;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < ncell;
         t += (long long)gridDim.x * blockDim.x) {
        const int x = 1 + (int)(t % nPx);
        const int y = 1 + (int)((t / nPx) % nPy);
        const int z = 1 + (int)(t / ((long long)nPx * nPy));
        const long long i = z * g.sz + y * g.sy + x;
        const double ro = U.p[S_RO][i], tt = U.p[S_TT][i];
        const double ru = U.p[S_RU][i], rv = U.p[S_RV][i], rw = U.p[S_RW][i];
        const double dv = c.DDX[x] * c.DDY[y] * c.DDZ[z];
        double e = 0.5 * (ru * ru + rv * rv + rw * rw) / ro + c.CV * ro * tt;
        int fl = 0;
        if (!(ro > 0.0)) fl |= 2;
        if (!(tt > 0.0)) fl |= 4;
        if constexpr (MAG) {
            const double bx = U.p[S_BX][i], by = U.p[S_BY][i], bz = U.p[S_BZ][i];
            e += 0.5 * c.OBETA * (bx * bx + by * by + bz * bz);
            if (z > 1 && z < g.nz - 2) {
                const double d = (U.p[S_BX][i + 1] - U.p[S_BX][i - 1]) * c.dxxdx[x] * c.hx +
                                 (U.p[S_BY][i + g.sy] - U.p[S_BY][i - g.sy]) * c.dyydy[y] * c.hy +
                                 (U.p[S_BZ][i + g.sz] - U.p[S_BZ][i - g.sz]) * c.dzzdz[z] * c.hz;
                divb = fmax(divb, fabs(d));
            }
            if (!isfinite(bx) || !isfinite(by) || !isfinite(bz)) fl |= 1;
        }
        if (!isfinite(ro) || !isfinite(tt) || !isfinite(ru) || !isfinite(rv) || !isfinite(rw)) fl |= 1;
        mass += ro * dv;
        energy += e * dv;
        flags = (double)((int)flags | fl);
    }
    __shared__ double s[4][kDiagThreads];
    s[0][threadIdx.x] = mass;
    s[1][threadIdx.x] = energy;
    s[2][threadIdx.x] = divb;
    s[3][threadIdx.x] = flags;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h) {
            s[0][threadIdx.x] += s[0][threadIdx.x + h];
            s[1][threadIdx.x] += s[1][threadIdx.x + h];
            s[2][threadIdx.x] = fmax(s[2][threadIdx.x], s[2][threadIdx.x + h]);
            s[3][threadIdx.x] = (double)((int)s[3][threadIdx.x] | (int)s[3][threadIdx.x + h]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int k = 0; k < 4; k++) part[(long long)k * gridDim.x + blockIdx.x] = s[k][0];
}

__global__ void k_diag_finish(const double* part, int nb, double* out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double m = 0, e = 0, d = 0;
    int f = 0;
    for (int b = 0; b < nb; b++) {
        m += part[b];
        e += part[nb + b];
        d = fmax(d, part[2LL * nb + b]);
        f |= (int)part[3LL * nb + b];
    }
    out[0] = m;
    out[1] = e;
    out[2] = d;
    out[3] = (double)f;
}

// Independent DFMA chains: the FP64 roof the fused kernel is measured against.
__global__ void k_fp64_peak(double* out, int iters, double a, double b) {
    double r[8];
#pragma unroll
    for (int k = 0; k < 8; k++) r[k] = threadIdx.x * 1e-9 + k;
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int k = 0; k < 8; k++) r[k] = fma(r[k], a, b);
    }
    double s = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) s += r[k];
    if (s == 1.2345) out[0] = s;  // keeps the chains live
}

}  // namespace

int fp64_peak(double* tflops) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    double* d = nullptr;
    if (cudaMalloc(&d, sizeof(double)) != cudaSuccess) return (int)cudaGetLastError();
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int threads = 256, blocks = sms * 8;
    // calibrate on a short run, then time one run of about 200 ms
    int iters = 32;
    float ms = 0.f;
    for (int pass = 0; pass < 2; pass++) {
        k_fp64_peak<<<blocks, threads>>>(d, 16, 0.999999, 1e-7);
        cudaEventRecord(e0);
        k_fp64_peak<<<blocks, threads>>>(d, iters, 0.999999, 1e-7);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
        if (pass == 0) {
            const double scale = 200.0 / (ms > 1e-3f ? ms : 1e-3f);
            iters = (int)(iters * scale);
            if (iters < 32) iters = 32;
            if (iters > 1 << 16) iters = 1 << 16;
        }
    }
    *tflops = 2.0 * 8.0 * iters * (double)blocks * threads / (ms * 1e-3) / 1e12;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(d);
    return (int)cudaGetLastError();
}

int diag_reduce(bool mag, const Grid& g, const Consts& c, Fields8 U, double* partials, int max_blocks, double* out4,
                cudaStream_t st) {
    const long long ncell = (long long)(g.nx - 2) * (g.ny - 2) * (g.nz - 2);
    long long nb = (ncell + kDiagThreads - 1) / kDiagThreads;
    if (nb > max_blocks) nb = max_blocks;
    if (nb < 1) nb = 1;
    if (mag) k_diag<true><<<(int)nb, kDiagThreads, 0, st>>>(g, c, U, partials);
    else k_diag<false><<<(int)nb, kDiagThreads, 0, st>>>(g, c, U, partials);
    k_diag_finish<<<1, 32, 0, st>>>(partials, (int)nb, out4);
    return (int)cudaGetLastError();
}

}  // namespace mhd
