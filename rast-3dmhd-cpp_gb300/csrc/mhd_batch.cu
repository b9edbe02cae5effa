// mhd_batch.cu -- many independent 3dmhd instances of uneven sizes stepped
// together: one persistent launch per RK3 substage over the ragged batch,
// the step captured in a CUDA graph, the tile shape chosen by an autotuner.
//
// Work list: every (instance, tile x, tile y, z range) of every instance, the
// longest z ranges first (longest processing time first: items of one tile
// shape cost in proportion to their planes); persistent CTAs take items from a
// counter (reset by a memset node at the start of each captured step), so
// instances of different sizes share the GPU without a launch per instance.
// The per-instance arguments of each substage live in a device array.  One
// step flips every instance's ping-pong buffers three times, so two graphs
// (even and odd step parity) are captured and launched alternately.
//
// Step limits: a device array left[i] holds the steps instance i still takes
// in the current call; the kernels skip the items of instances at 0 and a
// tick node at the end of every captured step decrements it.  So a call can
// step some instances fewer times than others (a server retires them when
// they reach their step count) without changing the captured graphs.
//
// Autotuner: for a batch signature (sizes, switch set, precision) not seen
// before, each candidate (tile shape, longest z range) is timed on a scratch
// copy of the batch's state (the real instances do not advance); the fastest
// is cached per signature.
#include "mhd_context.h"

#include <algorithm>
#include <cstdio>
#include <map>
#include <mutex>
#include <string>
#include <vector>

struct mhd_batch {
    std::vector<mhd_ctx*> ctx;
    std::vector<double> dt;
    unsigned sw = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int tile = -1;  // chosen tile shape
    int zmax = 64;  // longest z range of a work item (planes)
    bool uxy = true;   // every instance has uniform x/y grids
    bool fp32 = false; // FP32-storage instances (one tile shape, 32x8)
    int* d_left = nullptr;       // [n] steps each instance still takes in the current call
    int* d_err = nullptr;        // [4] the kernels' item checks (BatchCtl::err)
    int* h_left = nullptr;       // pinned staging of d_left
    cudaEvent_t left_copied = nullptr;  // the last copy of h_left has been read
    Fused32Args* d_args32 = nullptr;  // [2][3][n] for FP32 batches
    FusedArgs* d_args = nullptr;  // [2 parities][3 substages][n]
    int4* d_items = nullptr;
    int nitems = 0;
    int2* d_bitems = nullptr;
    int nbitems = 0;
    int* d_counters = nullptr;  // [2][3]
    int grid = 0;
    cudaGraphExec_t exec[2] = {nullptr, nullptr};
    int phase = 0;                // graph to launch next
    std::vector<int> expect_cur;  // each instance's cur when exec[phase] starts
    bool built = false;
    long long steps_done = 0;
    cudaEvent_t order = nullptr;  // orders the instances' streams around batch work
    std::string err;
};

namespace {

std::mutex g_tune_mutex;
std::map<std::string, std::pair<int, int>> g_tune_cache;  // signature -> (tile, zmax)

// Longest z range of a work item: the autotuner's second dimension.  Shorter
// ranges give more items (finer load balance over the persistent CTAs) but
// reload two halo planes each.
constexpr int kZChoices = 3;
constexpr int kZMax[kZChoices] = {64, 32, 16};
constexpr int kNoLimit = 1 << 30;

int bfail(mhd_batch* b, int code, const std::string& msg) {
    if (b) b->err = msg;
    fprintf(stderr, "mhd_batch: %s\n", msg.c_str());
    return code;
}

#define BCK(call)                                                                          \
    do {                                                                                   \
        cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess) return bfail(b, MHD_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

std::string signature(const mhd_batch* b) {
    std::vector<std::string> parts;
    for (const mhd_ctx* c : b->ctx)
        parts.push_back(std::to_string(c->g.nx) + "x" + std::to_string(c->g.ny) + "x" + std::to_string(c->g.nz));
    std::sort(parts.begin(), parts.end());
    std::string s = "sw" + std::to_string(b->sw) + (b->fp32 ? "f32" : "f64");
    for (auto& p : parts) s += "/" + p;
    return s;
}

// Per-instance arguments of every (parity, substage) given each instance's
// state buffers; U0/U1 may be a scratch copy (autotuner).
void fill_args(const mhd_batch* b, const std::vector<double*>& U0, const std::vector<double*>& U1,
               const std::vector<double*>& Z, const std::vector<double*>& FT, const std::vector<int>& cur0,
               std::vector<FusedArgs>& out) {
    const int n = (int)b->ctx.size();
    out.assign((size_t)6 * n, FusedArgs{});
    for (int p = 0; p < 2; p++)
        for (int s = 0; s < 3; s++)
            for (int i = 0; i < n; i++) {
                const mhd_ctx* c = b->ctx[i];
                const double gam[3] = {c->k.GAM1, c->k.GAM2, c->k.GAM3};
                const double zet[3] = {c->k.ZETA1, c->k.ZETA2, 0.0};
                const int cur = cur0[i] ^ ((3 * p + s) & 1);
                double* ubuf[2] = {U0[i], U1[i]};
                FusedArgs& a = out[((size_t)p * 3 + s) * n + i];
                a.g = c->g;
                a.c = c->c;
                a.k = c->coef;
                a.U = ctxops::fields_of(c, ubuf[cur]);
                a.Uo = ctxops::fields_of(c, ubuf[1 - cur]);
                a.Z = ctxops::fields_of(c, Z[i]);
                a.FT = FT[i];
                a.gdt = gam[s] * b->dt[i];
                a.zdt = zet[s] * b->dt[i];
                a.timt = c->timt;
                a.substage = s;
            }
}

// The same for FP32-storage instances; U0/U1 (FP32 state), Z and FT (FP64)
// may be a scratch copy (autotuner).
void fill_args32(const mhd_batch* b, const std::vector<float*>& U0, const std::vector<float*>& U1,
                 const std::vector<double*>& Z, const std::vector<double*>& FT, const std::vector<int>& cur0,
                 std::vector<Fused32Args>& out) {
    const int n = (int)b->ctx.size();
    out.assign((size_t)6 * n, Fused32Args{});
    for (int p = 0; p < 2; p++)
        for (int s = 0; s < 3; s++)
            for (int i = 0; i < n; i++) {
                const mhd_ctx* c = b->ctx[i];
                const double gam[3] = {c->k.GAM1, c->k.GAM2, c->k.GAM3};
                const double zet[3] = {c->k.ZETA1, c->k.ZETA2, 0.0};
                const int cur = cur0[i] ^ ((3 * p + s) & 1);
                const int nz = c->g.nz;
                float* ubuf[2] = {U0[i], U1[i]};
                Fused32Args& a = out[((size_t)p * 3 + s) * n + i];
                a.g = c->g;
                a.c = c->c;
                a.k = c->coef;
                a.U = ctxops::fields32_of(c, ubuf[cur]);
                a.Uo = ctxops::fields32_of(c, ubuf[1 - cur]);
                a.Z = ctxops::fields_of(c, Z[i]);
                a.FT = FT[i];
                a.bgR = c->d_bg;
                a.bgT = c->d_bg + nz;
                a.dzT0 = c->d_bg + 2 * nz;
                a.d2zT0 = c->d_bg + 3 * nz;
                a.zf = reinterpret_cast<const float*>(c->d_bg + 4 * nz);
                a.gdt = gam[s] * b->dt[i];
                a.zdt = zet[s] * b->dt[i];
                a.timt = c->timt;
                a.substage = s;
            }
}

// Work items for a tile shape and a longest z range: (instance, tile x,
// tile y, z range), the longest z ranges first.
void make_items(const mhd_batch* b, int tile, int zmax, std::vector<int4>& items) {
    int tx, ty;
    if (b->fp32) {
        tx = kBatch32TX;
        ty = kBatch32TY;
    } else {
        batch_tile_dims(tile, &tx, &ty);
    }
    items.clear();
    for (size_t i = 0; i < b->ctx.size(); i++) {
        const Grid& g = b->ctx[i]->g;
        const int nbx = (g.nx - 2 + tx - 1) / tx, nby = (g.ny - 2 + ty - 1) / ty;
        const int nPz = g.nz - 2, chunks = (nPz + zmax - 1) / zmax;
        for (int ch = 0; ch < chunks; ch++) {
            const int zb = 1 + nPz * ch / chunks, ze = 1 + nPz * (ch + 1) / chunks;
            for (int by = 0; by < nby; by++)
                for (int bx = 0; bx < nbx; bx++) items.push_back(make_int4((int)i, bx, by, zb | (ze << 16)));
        }
    }
    std::stable_sort(items.begin(), items.end(), [](const int4& a, const int4& c) {
        return ((a.w >> 16) - (a.w & 0xffff)) > ((c.w >> 16) - (c.w & 0xffff));
    });
}

// The kernels' item checks (batch_item_ok) on the host, before any capture:
// a malformed work list is reported as an error instead of being launched.
int check_items(mhd_batch* b, int tile, const std::vector<int4>& items) {
    int tx, ty;
    if (b->fp32) {
        tx = kBatch32TX;
        ty = kBatch32TY;
    } else {
        batch_tile_dims(tile, &tx, &ty);
    }
    const int n = (int)b->ctx.size();
    for (const int4& it : items) {
        const int zb = it.w & 0xffff, ze = it.w >> 16;
        bool ok = it.x >= 0 && it.x < n;
        if (ok) {
            const Grid& g = b->ctx[it.x]->g;
            ok = it.y >= 0 && it.z >= 0 && 1 + it.y * tx <= g.nx - 2 && 1 + it.z * ty <= g.ny - 2 && zb >= 1 &&
                 ze <= g.nz - 1 && zb < ze;
        }
        if (!ok)
            return bfail(b, MHD_ERR_INVALID, "malformed work item (instance " + std::to_string(it.x) + ", tile " +
                                                 std::to_string(it.y) + "," + std::to_string(it.z) + ", z " +
                                                 std::to_string(zb) + ".." + std::to_string(ze) + ")");
    }
    return MHD_OK;
}

void make_bcon_items(const mhd_batch* b, std::vector<int2>& items) {
    items.clear();
    for (size_t i = 0; i < b->ctx.size(); i++) {
        const Grid& g = b->ctx[i]->g;
        const int cells = 2 * (g.nx - 2) * (g.ny - 2);
        for (int s = 0; s < cells; s += 128) items.push_back(make_int2((int)i, s));
    }
}

int persistent_grid(mhd_batch* b, int tile, int nitems) {
    int dev = 0, sms = 0, per_sm = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int rc = b->fp32 ? fused32_batch_occupancy(b->sw, &per_sm)
                   : b->uxy ? fused_batch_occupancy_uxy(b->sw, tile, &per_sm)
                            : fused_batch_occupancy_gen(b->sw, tile, &per_sm);
    if (rc != 0 || per_sm < 1) per_sm = 1;
    return std::max(1, std::min(nitems, sms * per_sm));
}

// Capture the two step graphs for `tile` over the given argument array.
int capture(mhd_batch* b, int tile, const FusedArgs* d_args, const Fused32Args* d_args32, int4* d_items, int nitems,
            int* d_counters, cudaGraphExec_t out[2]) {
    const int n = (int)b->ctx.size();
    const int grid = persistent_grid(b, tile, nitems);
    const BatchCtl ctl{b->d_left, b->d_err, n};
    for (int p = 0; p < 2; p++) {
        cudaGraph_t graph;
        BCK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        cudaMemsetAsync(d_counters + 3 * p, 0, 3 * sizeof(int), b->stream);
        int rc = 0;
        for (int s = 0; s < 3 && !rc; s++) {
            if (b->fp32) {
                const Fused32Args* a32 = d_args32 + ((size_t)p * 3 + s) * n;
                rc = fused32_batch_substage(b->sw, a32, d_items, nitems, d_counters + 3 * p + s, ctl, grid,
                                            b->stream);
                if (!rc) rc = fused32_batch_bcon(b->sw, a32, b->d_bitems, ctl, b->nbitems, b->stream);
                continue;
            }
            const FusedArgs* args = d_args + ((size_t)p * 3 + s) * n;
            rc = b->uxy ? fused_batch_substage_uxy(b->sw, tile, args, d_items, nitems, d_counters + 3 * p + s,
                                                   ctl, grid, b->stream)
                        : fused_batch_substage_gen(b->sw, tile, args, d_items, nitems, d_counters + 3 * p + s,
                                                   ctl, grid, b->stream);
            if (!rc) rc = fused_batch_bcon(b->sw, args, b->d_bitems, ctl, b->nbitems, b->stream);
        }
        if (!rc) rc = batch_tick(b->d_left, n, b->stream);
        const cudaError_t ec = cudaStreamEndCapture(b->stream, &graph);
        if (rc || ec != cudaSuccess) return bfail(b, MHD_ERR_CUDA, "graph capture of the batched step failed");
        BCK(cudaGraphInstantiate(&out[p], graph, 0));
        cudaGraphDestroy(graph);
    }
    return MHD_OK;
}

void drop_graphs(cudaGraphExec_t e[2]) {
    for (int p = 0; p < 2; p++)
        if (e[p]) {
            cudaGraphExecDestroy(e[p]);
            e[p] = nullptr;
        }
}

// (Re)build the argument array, the work list and the graphs for the
// instances' current buffers.
int build(mhd_batch* b) {
    const int n = (int)b->ctx.size();
    std::vector<double*> U0(n), U1(n), Z(n), FT(n);
    std::vector<int> cur(n);
    for (int i = 0; i < n; i++) {
        mhd_ctx* c = b->ctx[i];
        int rc;
        if (b->fp32) {
            rc = ctxops::ensure_u32_1(c);
            if (!rc) rc = ctxops::sync_zghosts32(c);
        } else {
            rc = ctxops::ensure_u1(c);
            if (!rc && (c->sw & kSwShr)) rc = ctxops::alloc_block(c, &c->Fb, 8);
            if (!rc) rc = ctxops::sync_zghosts(c);
        }
        if (rc) return bfail(b, rc, "instance " + std::to_string(i) + ": " + c->err);
        BCK(cudaStreamSynchronize(c->stream));
        U0[i] = c->U[0];
        U1[i] = c->U[1];
        Z[i] = c->Zb;
        FT[i] = c->Fb ? c->Fb + (size_t)F_FT * c->ncell : nullptr;
        cur[i] = c->cur;
    }
    if (b->fp32) {
        std::vector<float*> V0(n), V1(n);
        std::vector<double*> Z32(n), FT32(n);
        for (int i = 0; i < n; i++) {
            V0[i] = b->ctx[i]->U32[0];
            V1[i] = b->ctx[i]->U32[1];
            Z32[i] = b->ctx[i]->Zb;
            FT32[i] = b->ctx[i]->FT64;
        }
        std::vector<Fused32Args> a32;
        fill_args32(b, V0, V1, Z32, FT32, cur, a32);
        BCK(cudaMemcpyAsync(b->d_args32, a32.data(), sizeof(Fused32Args) * a32.size(), cudaMemcpyHostToDevice,
                            b->stream));
        BCK(cudaStreamSynchronize(b->stream));
    } else {
        std::vector<FusedArgs> args;
        fill_args(b, U0, U1, Z, FT, cur, args);
        BCK(cudaMemcpyAsync(b->d_args, args.data(), sizeof(FusedArgs) * args.size(), cudaMemcpyHostToDevice, b->stream));
        BCK(cudaStreamSynchronize(b->stream));
    }
    std::vector<int4> items;
    make_items(b, b->tile, b->zmax, items);
    if (int rc = check_items(b, b->tile, items)) return rc;
    cudaFree(b->d_items);
    BCK(cudaMalloc(&b->d_items, sizeof(int4) * items.size()));
    // on the batch's stream, which the graphs run on: a plain cudaMemcpy runs on
    // the legacy stream, which the non-blocking batch stream does not wait for,
    // and its DMA may still be in flight when it returns
    BCK(cudaMemcpyAsync(b->d_items, items.data(), sizeof(int4) * items.size(), cudaMemcpyHostToDevice, b->stream));
    BCK(cudaStreamSynchronize(b->stream));
    b->nitems = (int)items.size();
    drop_graphs(b->exec);
    int rc = capture(b, b->tile, b->d_args, b->d_args32, b->d_items, b->nitems, b->d_counters, b->exec);
    if (rc) return rc;
    b->expect_cur = cur;
    b->phase = 0;
    b->built = true;
    return MHD_OK;
}

// Device bytes of the autotuner's scratch copy of the batch's state (FP64:
// U, U', Z and FT; FP32 storage: U, U' in FP32, Z and FT in FP64).
size_t tune_bytes(const mhd_batch* b) {
    size_t t = 0;
    for (const mhd_ctx* c : b->ctx) {
        const size_t ft = (c->sw & kSwShr) ? 1 : 0;
        t += b->fp32 ? c->ncell * (16 * sizeof(float) + (8 + ft) * sizeof(double))
                     : c->ncell * (24 + ft) * sizeof(double);
    }
    return t;
}

// Time every (tile shape, longest z range) on a scratch copy of the batch;
// returns the fastest as tile + kBatchTiles * z choice.  ms_out[t]: the best
// time per step of tile t (0 for tiles that were not candidates).
int autotune(mhd_batch* b, double* ms_out) {
    const int n = (int)b->ctx.size();
    std::vector<double*> U0(n), U1(n), Z(n), FT(n);
    std::vector<float*> V0(n), V1(n);
    std::vector<void*> owned;
    std::vector<int> cur(n, 0);
    int rc = MHD_OK;
    for (int i = 0; i < n && !rc; i++) {
        mhd_ctx* c = b->ctx[i];
        const size_t fb = c->ncell * sizeof(double);
        const int nf_ft = (c->sw & kSwShr) ? 1 : 0;
        const size_t nb = b->fp32 ? c->ncell * 16 * sizeof(float) + fb * (8 + nf_ft) : fb * (24 + nf_ft);
        unsigned char* blk = nullptr;
        if (cudaMalloc(&blk, nb) != cudaSuccess) {
            cudaGetLastError();
            rc = bfail(b, MHD_ERR_NOMEM, "autotuner scratch allocation failed");
            break;
        }
        owned.push_back(blk);
        if (b->fp32) {
            V0[i] = reinterpret_cast<float*>(blk);
            V1[i] = V0[i] + 8 * c->ncell;
            Z[i] = reinterpret_cast<double*>(blk + c->ncell * 16 * sizeof(float));
            FT[i] = nf_ft ? Z[i] + 8 * c->ncell : nullptr;
            cudaMemcpyAsync(V0[i], c->U32[c->cur], c->ncell * 8 * sizeof(float), cudaMemcpyDeviceToDevice, b->stream);
            cudaMemcpyAsync(V1[i], c->U32[c->cur], c->ncell * 8 * sizeof(float), cudaMemcpyDeviceToDevice, b->stream);
            cudaMemcpyAsync(Z[i], c->Zb, fb * 8, cudaMemcpyDeviceToDevice, b->stream);
        } else {
            U0[i] = reinterpret_cast<double*>(blk);
            U1[i] = U0[i] + 8 * c->ncell;
            Z[i] = U0[i] + 16 * c->ncell;
            FT[i] = nf_ft ? U0[i] + 24 * c->ncell : nullptr;
            cudaMemcpyAsync(U0[i], c->U[c->cur], fb * 8, cudaMemcpyDeviceToDevice, b->stream);
            cudaMemcpyAsync(U1[i], c->U[c->cur], fb * 8, cudaMemcpyDeviceToDevice, b->stream);
            cudaMemsetAsync(Z[i], 0, fb * 8, b->stream);
        }
        if (FT[i]) cudaMemsetAsync(FT[i], 0, fb, b->stream);
    }
    FusedArgs* d_args = nullptr;
    Fused32Args* d_args32 = nullptr;
    int* d_cnt = nullptr;
    int best = 0;
    double best_ms = 1e300;
    if (!rc && cudaMalloc(&d_args, sizeof(FusedArgs) * 6 * n) != cudaSuccess) rc = MHD_ERR_NOMEM;
    if (!rc && cudaMalloc(&d_args32, sizeof(Fused32Args) * 6 * n) != cudaSuccess) rc = MHD_ERR_NOMEM;
    if (!rc && cudaMalloc(&d_cnt, sizeof(int) * 6) != cudaSuccess) rc = MHD_ERR_NOMEM;
    if (!rc) {
        if (b->fp32) {
            std::vector<Fused32Args> a32;
            fill_args32(b, V0, V1, Z, FT, cur, a32);
            cudaMemcpyAsync(d_args32, a32.data(), sizeof(Fused32Args) * a32.size(), cudaMemcpyHostToDevice, b->stream);
            cudaStreamSynchronize(b->stream);
        } else {
            std::vector<FusedArgs> args;
            fill_args(b, U0, U1, Z, FT, cur, args);
            cudaMemcpyAsync(d_args, args.data(), sizeof(FusedArgs) * args.size(), cudaMemcpyHostToDevice, b->stream);
            cudaStreamSynchronize(b->stream);
        }
        // every instance steps in every timed step (the staging buffer is reused:
        // a call's steps may still be waiting to read it)
        cudaEventSynchronize(b->left_copied);
        for (int i = 0; i < n; i++) b->h_left[i] = kNoLimit;
        cudaMemcpyAsync(b->d_left, b->h_left, sizeof(int) * n, cudaMemcpyHostToDevice, b->stream);
        cudaEventRecord(b->left_copied, b->stream);
        if (ms_out)
            for (int t = 0; t < kBatchTiles; t++) ms_out[t] = 0.0;
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        const int ntiles = b->fp32 ? 1 : kBatchTiles;
        for (int cand = 0; cand < ntiles * kZChoices && !rc; cand++) {
            const int t = cand % ntiles, zc = cand / ntiles;
            std::vector<int4> items;
            make_items(b, t, kZMax[zc], items);
            if ((rc = check_items(b, t, items))) break;
            int4* d_items = nullptr;
            if (cudaMalloc(&d_items, sizeof(int4) * items.size()) != cudaSuccess) {
                rc = MHD_ERR_NOMEM;
                break;
            }
            cudaMemcpyAsync(d_items, items.data(), sizeof(int4) * items.size(), cudaMemcpyHostToDevice, b->stream);
            cudaStreamSynchronize(b->stream);
            cudaGraphExec_t ex[2] = {nullptr, nullptr};
            rc = capture(b, t, d_args, d_args32, d_items, (int)items.size(), d_cnt, ex);
            if (!rc) {
                for (int w = 0; w < 2; w++) cudaGraphLaunch(ex[w], b->stream);
                cudaEventRecord(e0, b->stream);
                const int reps = 4;
                for (int r = 0; r < reps; r++) cudaGraphLaunch(ex[r & 1], b->stream);
                cudaEventRecord(e1, b->stream);
                cudaEventSynchronize(e1);
                float ms = 0.f;
                cudaEventElapsedTime(&ms, e0, e1);
                const double per = ms / reps;
                if (ms_out && (ms_out[t] == 0.0 || per < ms_out[t])) ms_out[t] = per;
                if (per < best_ms) {
                    best_ms = per;
                    best = t + kBatchTiles * zc;
                }
            }
            drop_graphs(ex);
            cudaFree(d_items);
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
    }
    cudaStreamSynchronize(b->stream);
    cudaFree(d_args);
    cudaFree(d_args32);
    cudaFree(d_cnt);
    for (void* p : owned) cudaFree(p);
    if (rc) return rc;
    return best;
}

}  // namespace

extern "C" {

int mhd_batch_create(mhd_ctx* const* ctxs, const double* dts, int n, void* stream, mhd_batch** out) {
    if (!out || !ctxs || !dts || n <= 0) return MHD_ERR_INVALID;
    *out = nullptr;
    mhd_batch* b = new mhd_batch();
    for (int i = 0; i < n; i++) {
        mhd_ctx* c = ctxs[i];
        if (!c || !(dts[i] > 0.0)) {
            delete b;
            return MHD_ERR_INVALID;
        }
        if (c->prm.path != MHD_PATH_FUSED) {
            delete b;
            fprintf(stderr, "mhd_batch_create: instances must be fused-path contexts\n");
            return MHD_ERR_UNSUPPORTED;
        }
        if (c->c.lrem) {
            delete b;
            fprintf(stderr, "mhd_batch_create: lRem instances step alone (per-substage plane means)\n");
            return MHD_ERR_UNSUPPORTED;
        }
        if (c->c.pl_mode == 3 || (c->c.pl_mode != 0 && (!c->plume_set || ctxops::plume_time_dependent(c)))) {
            delete b;
            fprintf(stderr, "mhd_batch_create: batched instances may carry only a time-independent top-wall plume "
                            "(TC = 0); the iTCon 2 heat sink steps alone\n");
            return MHD_ERR_UNSUPPORTED;
        }
        if (i > 0 && (c->sw != b->sw || c->fp32 != b->fp32)) {
            delete b;
            fprintf(stderr, "mhd_batch_create: all instances of a batch need the same switch set\n");
            return MHD_ERR_UNSUPPORTED;
        }
        b->sw = c->sw;
        b->fp32 = c->fp32;
        b->uxy = b->uxy && c->coef.uniform_xy;
        b->ctx.push_back(c);
        b->dt.push_back(dts[i]);
    }
    if (stream) {
        b->stream = (cudaStream_t)stream;
    } else if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) == cudaSuccess) {
        b->own_stream = true;
    } else {
        delete b;
        return MHD_ERR_CUDA;
    }
    std::vector<int2> bitems;
    make_bcon_items(b, bitems);
    b->nbitems = (int)bitems.size();
    if (cudaMalloc(&b->d_args, sizeof(FusedArgs) * 6 * n) != cudaSuccess ||
        cudaMalloc(&b->d_args32, sizeof(Fused32Args) * 6 * n) != cudaSuccess ||
        cudaMalloc(&b->d_counters, sizeof(int) * 6) != cudaSuccess ||
        cudaMalloc(&b->d_bitems, sizeof(int2) * bitems.size()) != cudaSuccess ||
        cudaMemcpyAsync(b->d_bitems, bitems.data(), sizeof(int2) * bitems.size(), cudaMemcpyHostToDevice, b->stream) !=
            cudaSuccess ||
        cudaMalloc(&b->d_left, sizeof(int) * n) != cudaSuccess ||
        cudaMalloc(&b->d_err, sizeof(int) * 4) != cudaSuccess ||
        cudaMemsetAsync(b->d_err, 0, sizeof(int) * 4, b->stream) != cudaSuccess ||
        cudaStreamSynchronize(b->stream) != cudaSuccess ||
        cudaMallocHost(&b->h_left, sizeof(int) * n) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->left_copied, cudaEventDisableTiming) != cudaSuccess) {
        cudaGetLastError();
        mhd_batch_destroy(b);
        return MHD_ERR_NOMEM;
    }
    *out = b;
    return MHD_OK;
}

int mhd_batch_destroy(mhd_batch* b) {
    if (!b) return MHD_ERR_INVALID;
    if (b->stream) cudaStreamSynchronize(b->stream);
    drop_graphs(b->exec);
    if (b->order) cudaEventDestroy(b->order);
    if (b->left_copied) cudaEventDestroy(b->left_copied);
    cudaFree(b->d_args);
    cudaFree(b->d_args32);
    cudaFree(b->d_items);
    cudaFree(b->d_bitems);
    cudaFree(b->d_counters);
    cudaFree(b->d_left);
    cudaFree(b->d_err);
    if (b->h_left) cudaFreeHost(b->h_left);
    if (b->own_stream) cudaStreamDestroy(b->stream);
    delete b;
    return MHD_OK;
}

int mhd_batch_set_tile(mhd_batch* b, int tile) {
    if (!b || tile < -1 || tile >= kBatchTiles) return MHD_ERR_INVALID;
    if (b->fp32 && tile > 0) return MHD_ERR_INVALID;  // one tile shape (32x8) for FP32 storage
    b->tile = tile;
    b->built = false;
    return MHD_OK;
}

int mhd_batch_set_zrange(mhd_batch* b, int zmax) {
    if (!b || zmax < 1 || zmax > 4096) return MHD_ERR_INVALID;
    b->zmax = zmax;
    b->built = false;
    return MHD_OK;
}

int mhd_batch_zrange(const mhd_batch* b, int* zmax) {
    if (!b || !zmax) return MHD_ERR_INVALID;
    *zmax = b->zmax;
    return MHD_OK;
}

int mhd_batch_autotune_bytes(const mhd_batch* b, unsigned long long* bytes) {
    if (!b || !bytes) return MHD_ERR_INVALID;
    *bytes = (unsigned long long)tune_bytes(b);
    return MHD_OK;
}

int mhd_batch_autotune(mhd_batch* b, int* chosen, double* ms_per_step) {
    if (!b) return MHD_ERR_INVALID;
    const std::string sig = signature(b);
    int best_tile = -1, best_z = 64;
    if (!ms_per_step) {
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        auto it = g_tune_cache.find(sig);
        if (it != g_tune_cache.end()) {
            best_tile = it->second.first;
            best_z = it->second.second;
        }
    }
    if (best_tile < 0) {
        const int best = autotune(b, ms_per_step);
        if (best < 0) return best;
        best_tile = best % kBatchTiles;
        best_z = kZMax[best / kBatchTiles];
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        g_tune_cache[sig] = {best_tile, best_z};
    }
    b->tile = best_tile;
    b->zmax = best_z;
    b->built = false;
    if (chosen) *chosen = best_tile;
    return MHD_OK;
}

namespace {

// Queue nsteps batched steps; instance i takes min(nsteps, limits[i]) of them
// (all of them when limits is null).
int batch_steps(mhd_batch* b, int nsteps, const int* limits) {
    if (!b || nsteps < 0) return MHD_ERR_INVALID;
    const int n = (int)b->ctx.size();
    if (limits)
        for (int i = 0; i < n; i++)
            if (limits[i] < 0) return MHD_ERR_INVALID;
    if (b->tile < 0) {
        int rc = mhd_batch_autotune(b, nullptr, nullptr);
        if (rc) return rc;
    }
    bool stale = !b->built;
    for (int i = 0; i < n && !stale; i++)
        stale = b->ctx[i]->cur != b->expect_cur[i] || !b->ctx[i]->ghosts_synced;
    if (stale) {
        int rc = build(b);
        if (rc) return rc;
    }
    if (nsteps == 0) return MHD_OK;
    if (!b->order) BCK(cudaEventCreateWithFlags(&b->order, cudaEventDisableTiming));
    // the staging buffer is reused: wait until the previous call's copy has read it
    BCK(cudaEventSynchronize(b->left_copied));
    for (int i = 0; i < n; i++) b->h_left[i] = limits ? std::min(limits[i], nsteps) : kNoLimit;
    // work queued on the instances' own streams (uploads, single steps) first
    for (mhd_ctx* c : b->ctx) {
        BCK(cudaEventRecord(b->order, c->stream));
        BCK(cudaStreamWaitEvent(b->stream, b->order, 0));
    }
    BCK(cudaMemcpyAsync(b->d_left, b->h_left, sizeof(int) * n, cudaMemcpyHostToDevice, b->stream));
    BCK(cudaEventRecord(b->left_copied, b->stream));
    for (int s = 0; s < nsteps; s++) {
        BCK(cudaGraphLaunch(b->exec[b->phase], b->stream));
        b->phase ^= 1;
        for (int i = 0; i < n; i++) {
            mhd_ctx* c = b->ctx[i];
            b->expect_cur[i] ^= 1;  // what the graphs assume
            if (!limits || s < limits[i]) {
                c->cur ^= 1;
                ctxops::advance_time(c, b->dt[i]);
            }
        }
        b->steps_done++;
    }
    // later work on an instance's stream (downloads, diagnostics) waits for the batch
    BCK(cudaEventRecord(b->order, b->stream));
    for (mhd_ctx* c : b->ctx) BCK(cudaStreamWaitEvent(c->stream, b->order, 0));
    return MHD_OK;
}

}  // namespace

int mhd_batch_steps(mhd_batch* b, int nsteps) { return batch_steps(b, nsteps, nullptr); }

int mhd_batch_steps_limited(mhd_batch* b, int nsteps, const int* max_steps) {
    if (!max_steps) return MHD_ERR_INVALID;
    return batch_steps(b, nsteps, max_steps);
}

int mhd_batch_sync(mhd_batch* b) {
    if (!b) return MHD_ERR_INVALID;
    BCK(cudaStreamSynchronize(b->stream));
    // the kernels' work-item checks: a failed item was skipped, not stepped
    int e[4] = {0, 0, 0, 0};
    BCK(cudaMemcpy(e, b->d_err, sizeof(e), cudaMemcpyDeviceToHost));
    if (e[0])
        return bfail(b, MHD_ERR_INVALID,
                     "a work item failed its check (code " + std::to_string(e[0]) + ", instance " +
                         std::to_string(e[1]) + ", tile " + std::to_string(e[2] & 0xffff) + "," +
                         std::to_string(e[2] >> 16) + ", z " + std::to_string(e[3] & 0xffff) + ".." +
                         std::to_string(e[3] >> 16) + ") and was skipped");
    return MHD_OK;
}

int mhd_batch_tile(const mhd_batch* b, int* tile) {
    if (!b || !tile) return MHD_ERR_INVALID;
    *tile = b->tile;
    return MHD_OK;
}

}  // extern "C"
