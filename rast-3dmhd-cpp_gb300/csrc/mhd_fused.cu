// mhd_fused.cu -- launches of the fused FP64 RK3 substage for one instance
// (the per-tile work is in mhd_fused_tile.cuh) and of the wall kernel.
//
// The grid is (x tiles, y tiles, z chunks): splitting every column into a few
// z ranges turns the tail wave of a large grid into many short work units.
// The number of chunks minimises (waves needed / waves of work) x (planes
// loaded / planes computed) for the occupancy the device reports.
#include "mhd_fused_tile.cuh"

#include <cmath>

namespace mhd {
namespace {

using namespace fused;
// tile of the single-instance kernel (MHD_FUSED_TILE_X x MHD_FUSED_TILE_Y threads):
// 16 x 8 loads 18 x 10 ring points per 128 cells (32 x 4: 34 x 6), and each
// warp still reads whole 128-byte rows (measured: 71.7 vs 72.9 ms per step at
// 512 x 512 x 256; 32 x 6, 32 x 8 and 16 x 12 run fewer CTAs per SM and are slower)
#ifndef MHD_FUSED_TILE_X
#define MHD_FUSED_TILE_X 16
#endif
#ifndef MHD_FUSED_TILE_Y
#define MHD_FUSED_TILE_Y 8
#endif
// This file is compiled twice: MHD_FUSED_XP=0 gives the kernels without the
// optional temperature terms (and the dispatcher and the wall kernels),
// MHD_FUSED_XP=1 the ones with the iTCon 2 heat sink and lRem.
#ifndef MHD_FUSED_XP
#define MHD_FUSED_XP 0
#endif
constexpr bool kExtra = MHD_FUSED_XP != 0;
using DefaultTile = Tile<MHD_FUSED_TILE_X, MHD_FUSED_TILE_Y>;
constexpr int kMinBlocks = DefaultTile::kThreads >= 256 ? 2 : 3;

template <class SW, bool UXY, bool ISO>
__global__ void __launch_bounds__(DefaultTile::kThreads, kMinBlocks) k_substage(FusedArgs a) {
    extern __shared__ double ring[];
    const int lo = a.zhi > 0 ? a.zlo : 1;
    const int nz = (a.zhi > 0 ? a.zhi : a.g.nz - 1) - lo;
    const int zb = lo + (int)((long long)nz * blockIdx.z / gridDim.z);
    const int ze = lo + (int)((long long)nz * (blockIdx.z + 1) / gridDim.z);
    substage_tile<SW, DefaultTile, UXY, kExtra, ISO>(a, blockIdx.x, blockIdx.y, zb, ze, ring);
}

template <class SW>
__global__ void k_bcon_ghost(Grid g, Consts c, Fields8 U, double timt, int wall0, int nwalls) {
    const int nPx = g.nx - 2, nPy = g.ny - 2;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nwalls * nPx * nPy) return;
    const int r = t % (nPx * nPy);
    bcon_cell<SW>(g, c, U, timt, wall0 + t / (nPx * nPy), 1 + r % nPx, 1 + r / nPx);
}

int choose_chunks(long long tiles, int slots, int nPz) {
    int best = 1;
    double best_cost = 1e300;
    for (int c = 1; c <= 8 && c <= nPz / 4; c++) {
        const double units = (double)tiles * c;
        const double waves = std::ceil(units / slots);
        const double eff = units / (waves * slots);
        const double cost = (1.0 + 2.0 * c / nPz) / eff;
        if (cost < best_cost - 1e-9) {
            best_cost = cost;
            best = c;
        }
    }
    return best;
}

template <class SW, bool UXY, bool ISO>
int launch_t(const FusedArgs& a, cudaStream_t st) {
    using T = DefaultTile;
    const size_t smem = ring_bytes<SW, T>();
    static int slots = 0;
    if (!slots) {
        cudaFuncSetAttribute(k_substage<SW, UXY, ISO>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        int dev = 0, sms = 0, per_sm = 1;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_substage<SW, UXY, ISO>, T::kThreads, smem);
        slots = sms * (per_sm > 0 ? per_sm : 1);
    }
    const int nbx = (a.g.nx - 2 + T::kTX - 1) / T::kTX, nby = (a.g.ny - 2 + T::kTY - 1) / T::kTY;
    const int planes = a.zhi > 0 ? a.zhi - a.zlo : a.g.nz - 2;
    const int chunks = choose_chunks((long long)nbx * nby, slots, planes);
    k_substage<SW, UXY, ISO><<<dim3(nbx, nby, chunks), T::kThreads, smem, st>>>(a);
    return (int)cudaGetLastError();
}

template <class SW>
void launch_substage(const FusedArgs& a, cudaStream_t st, int* rc) {
    // the instantiation with the optional temperature terms has no isotropic variant
    if (!kExtra && a.k.uniform_xy && a.k.isotropic_xy) *rc = launch_t<SW, true, !kExtra>(a, st);
    else *rc = a.k.uniform_xy ? launch_t<SW, true, false>(a, st) : launch_t<SW, false, false>(a, st);
}

template <class SW>
void launch_bcon_ghost(const Grid& g, const Consts& c, Fields8 U, double timt, int wall, cudaStream_t st) {
    const int nwalls = wall < 0 ? 2 : 1, wall0 = wall < 0 ? 0 : wall;
    const int n = nwalls * (g.nx - 2) * (g.ny - 2);
    k_bcon_ghost<SW><<<(n + 127) / 128, 128, 0, st>>>(g, c, U, timt, wall0, nwalls);
}

}  // namespace

#if MHD_FUSED_XP
int fused_substage_xp(unsigned sw, const FusedArgs& a, cudaStream_t st) {
    int rc = 0;
    MHD_DISPATCH_SW(sw, launch_substage, a, st, &rc);
    return rc;
}
#else
int fused_substage(unsigned sw, const FusedArgs& a, cudaStream_t st) {
    if (a.c.pl_mode == 3 || a.c.lrem) return fused_substage_xp(sw, a, st);
    int rc = 0;
    MHD_DISPATCH_SW(sw, launch_substage, a, st, &rc);
    return rc;
}

int fused_bcon_ghost(unsigned sw, const Grid& g, const Consts& c, Fields8 U, double timt, cudaStream_t st) {
    MHD_DISPATCH_SW(sw, launch_bcon_ghost, g, c, U, timt, -1, st);
    return (int)cudaGetLastError();
}

int fused_bcon_wall(unsigned sw, const Grid& g, const Consts& c, Fields8 U, double timt, int wall, cudaStream_t st) {
    MHD_DISPATCH_SW(sw, launch_bcon_ghost, g, c, U, timt, wall, st);
    return (int)cudaGetLastError();
}
#endif

}  // namespace mhd
