// mhd_fused_batch.cu -- the fused FP64 substage over a ragged batch of
// instances: persistent CTAs take (instance, tile x, tile y, z range) work
// items from a counter until none are left, so instances of different sizes
// share one launch.  Built twice: MHD_BATCH_UXY = 1 for uniform x/y grids
// (with the isotropic variant chosen per work item), 0 for stretched ones;
// the tile shapes are the autotuner's candidates.
#include "mhd_fused_tile.cuh"

#ifndef MHD_BATCH_UXY
#define MHD_BATCH_UXY 0
#endif

namespace mhd {
namespace {

using namespace fused;
constexpr bool kUXY = MHD_BATCH_UXY != 0;
using BatchTile0 = Tile<32, 4>;
using BatchTile1 = Tile<32, 8>;
using BatchTile2 = Tile<16, 8>;

// item: x = instance, y = tile x, z = tile y, w = first z plane | end plane << 16.
// ctl.left[i]: steps instance i still takes in this call (items of an
// instance at 0 are skipped, so instances that finish early drop out of the
// work); items that fail batch_item_ok are recorded in ctl.err and skipped.
template <class SW, class T>
__global__ void __launch_bounds__(T::kThreads) k_substage_batch(const FusedArgs* __restrict__ args,
                                                                const int4* __restrict__ items, int nitems,
                                                                int* counter, BatchCtl ctl) {
    extern __shared__ double ring[];
    __shared__ int s_item;
    for (;;) {
        if (threadIdx.x == 0) s_item = atomicAdd(counter, 1);
        __syncthreads();
        const int t = s_item;
        __syncthreads();
        if (t >= nitems) break;
        const int4 it = items[t];
        // both tests are uniform over the CTA
        if (!batch_item_ok(ctl, args, it, T::kTX, T::kTY, SW::lMag ? 8 : 5) || ctl.left[it.x] <= 0) continue;
        const FusedArgs& a = args[it.x];
        // each instance runs the variant it runs alone (isotropic or not), so
        // a batch reproduces its instances' single-instance results bit for bit
        if (kUXY && a.k.isotropic_xy) substage_tile<SW, T, kUXY, false, kUXY>(a, it.y, it.z, it.w & 0xffff, it.w >> 16, ring);
        else substage_tile<SW, T, kUXY>(a, it.y, it.z, it.w & 0xffff, it.w >> 16, ring);
        __syncthreads();
    }
}

// BCON for a ragged batch: block b covers 128 wall cells of instance items[b].x
// starting at cell items[b].y.
template <class SW>
__global__ void k_bcon_ghost_batch(const FusedArgs* __restrict__ args, const int2* __restrict__ items, BatchCtl ctl) {
    const int2 it = items[blockIdx.x];
    if (it.x < 0 || it.x >= ctl.n) {
        if (threadIdx.x == 0 && atomicCAS(ctl.err, 0, 1) == 0) ctl.err[1] = it.x;
        return;
    }
    if (ctl.left[it.x] <= 0) return;
    const FusedArgs& a = args[it.x];
    const int nPx = a.g.nx - 2, nPy = a.g.ny - 2;
    const int t = it.y + threadIdx.x;
    if (t >= 2 * nPx * nPy) return;
    const int r = t % (nPx * nPy);
    bcon_cell<SW>(a.g, a.c, a.Uo, a.timt, t / (nPx * nPy), 1 + r % nPx, 1 + r / nPx);
}

template <class SW, class T>
int batch_launch_t(const FusedArgs* args, const int4* items, int nitems, int* counter, BatchCtl ctl, int grid,
                   cudaStream_t st) {
    // the shared-memory attribute is set by batch_occupancy_t, which runs before any capture
    const size_t smem = ring_bytes<SW, T>();
    k_substage_batch<SW, T><<<grid, T::kThreads, smem, st>>>(args, items, nitems, counter, ctl);
    return (int)cudaGetLastError();
}

template <class SW, class T>
int batch_occupancy_t(int* blocks) {
    const size_t smem = ring_bytes<SW, T>();
    cudaFuncSetAttribute(k_substage_batch<SW, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    return (int)cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, k_substage_batch<SW, T>, T::kThreads, smem);
}

template <class SW>
void batch_launch_sw(int tile, const FusedArgs* args, const int4* items, int nitems, int* counter, BatchCtl ctl,
                     int grid, cudaStream_t st, int* rc) {
    if (tile == 0) *rc = batch_launch_t<SW, BatchTile0>(args, items, nitems, counter, ctl, grid, st);
    else if (tile == 1) *rc = batch_launch_t<SW, BatchTile1>(args, items, nitems, counter, ctl, grid, st);
    else *rc = batch_launch_t<SW, BatchTile2>(args, items, nitems, counter, ctl, grid, st);
}

template <class SW>
void batch_occupancy_sw(int tile, int* blocks, int* rc) {
    if (tile == 0) *rc = batch_occupancy_t<SW, BatchTile0>(blocks);
    else if (tile == 1) *rc = batch_occupancy_t<SW, BatchTile1>(blocks);
    else *rc = batch_occupancy_t<SW, BatchTile2>(blocks);
}

template <class SW>
void batch_bcon_sw(const FusedArgs* args, const int2* items, BatchCtl ctl, int nblocks, cudaStream_t st) {
    k_bcon_ghost_batch<SW><<<nblocks, 128, 0, st>>>(args, items, ctl);
}

// end of a batched step: one step fewer left for every instance still stepping
__global__ void k_batch_tick(int* left, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && left[i] > 0) left[i] -= 1;
}

}  // namespace

#if MHD_BATCH_UXY
#define MHD_BATCH_FN(name) name##_uxy
#else
#define MHD_BATCH_FN(name) name##_gen
#endif

int MHD_BATCH_FN(fused_batch_substage)(unsigned sw, int tile, const FusedArgs* args, const int4* items, int nitems,
                                       int* counter, BatchCtl ctl, int grid, cudaStream_t st) {
    int rc = 0;
    MHD_DISPATCH_SW(sw, batch_launch_sw, tile, args, items, nitems, counter, ctl, grid, st, &rc);
    return rc;
}

int MHD_BATCH_FN(fused_batch_occupancy)(unsigned sw, int tile, int* blocks_per_sm) {
    int rc = 0;
    MHD_DISPATCH_SW(sw, batch_occupancy_sw, tile, blocks_per_sm, &rc);
    return rc;
}

#if MHD_BATCH_UXY
// the wall kernel does not depend on the grid kind: built once
int fused_batch_bcon(unsigned sw, const FusedArgs* args, const int2* items, BatchCtl ctl, int nblocks,
                     cudaStream_t st) {
    MHD_DISPATCH_SW(sw, batch_bcon_sw, args, items, ctl, nblocks, st);
    return (int)cudaGetLastError();
}

int batch_tick(int* left, int n, cudaStream_t st) {
    k_batch_tick<<<(n + 255) / 256, 256, 0, st>>>(left, n);
    return (int)cudaGetLastError();
}

void batch_tile_dims(int tile, int* tx, int* ty) {
    static const int d[3][2] = {{32, 4}, {32, 8}, {16, 8}};
    *tx = d[tile][0];
    *ty = d[tile][1];
}
#endif

}  // namespace mhd
