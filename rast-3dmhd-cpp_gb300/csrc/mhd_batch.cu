// mhd_batch.cu -- many independent 3dmhd instances of uneven sizes stepped
// together: one persistent launch per RK3 substage over the ragged batch,
// the step captured in a CUDA graph, the tile shape chosen by an autotuner.
//
// Work list: every (instance, tile x, tile y) of every instance, largest z
// extent first; persistent CTAs take items from a counter (reset by a memset
// node at the start of each captured step), so instances of different sizes
// share the GPU without a launch per instance.  The per-instance arguments of
// each substage live in a device array.  One step flips every instance's
// ping-pong buffers three times, so two graphs (even and odd step parity) are
// captured and launched alternately.
//
// Autotuner: for a batch signature (sizes, switch set) not seen before, each
// candidate tile shape is timed on a scratch copy of the batch's state (the
// real instances do not advance); the fastest is cached per signature.
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
    bool uxy = true;   // every instance has uniform x/y grids
    bool fp32 = false; // FP32-storage instances (one tile shape, 32x8)
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
std::map<std::string, int> g_tune_cache;

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
    std::string s = "sw" + std::to_string(b->sw);
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

void fill_args32(const mhd_batch* b, const std::vector<int>& cur0, std::vector<Fused32Args>& out) {
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
                Fused32Args& a = out[((size_t)p * 3 + s) * n + i];
                a.g = c->g;
                a.c = c->c;
                a.k = c->coef;
                a.U = ctxops::fields32_of(c, c->U32[cur]);
                a.Uo = ctxops::fields32_of(c, c->U32[1 - cur]);
                a.Z = ctxops::fields_of(c, c->Zb);
                a.FT = c->FT64;
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

// Work items for a tile shape: (instance, tile x, tile y), largest z first.
void make_items(const mhd_batch* b, int tile, std::vector<int4>& items) {
    int tx, ty;
    if (b->fp32) {
        tx = kBatch32TX;
        ty = kBatch32TY;
    } else {
        batch_tile_dims(tile, &tx, &ty);
    }
    std::vector<int> order(b->ctx.size());
    for (size_t i = 0; i < order.size(); i++) order[i] = (int)i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int c) {
        const Grid &ga = b->ctx[a]->g, &gc = b->ctx[c]->g;
        return (long long)ga.nz > (long long)gc.nz;
    });
    items.clear();
    for (int i : order) {
        const Grid& g = b->ctx[i]->g;
        const int nbx = (g.nx - 2 + tx - 1) / tx, nby = (g.ny - 2 + ty - 1) / ty;
        const int nPz = g.nz - 2, chunks = (nPz + 63) / 64;  // z ranges of at most 64 planes
        for (int ch = 0; ch < chunks; ch++) {
            const int zb = 1 + nPz * ch / chunks, ze = 1 + nPz * (ch + 1) / chunks;
            for (int by = 0; by < nby; by++)
                for (int bx = 0; bx < nbx; bx++) items.push_back(make_int4(i, bx, by, zb | (ze << 16)));
        }
    }
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
int capture(mhd_batch* b, int tile, FusedArgs* d_args, int4* d_items, int nitems, int* d_counters,
            cudaGraphExec_t out[2]) {
    const int n = (int)b->ctx.size();
    const int grid = persistent_grid(b, tile, nitems);
    for (int p = 0; p < 2; p++) {
        cudaGraph_t graph;
        BCK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        cudaMemsetAsync(d_counters + 3 * p, 0, 3 * sizeof(int), b->stream);
        int rc = 0;
        for (int s = 0; s < 3 && !rc; s++) {
            if (b->fp32) {
                const Fused32Args* a32 = b->d_args32 + ((size_t)p * 3 + s) * n;
                rc = fused32_batch_substage(b->sw, a32, d_items, nitems, d_counters + 3 * p + s, grid, b->stream);
                if (!rc) rc = fused32_batch_bcon(b->sw, a32, b->d_bitems, b->nbitems, b->stream);
                continue;
            }
            const FusedArgs* args = d_args + ((size_t)p * 3 + s) * n;
            rc = b->uxy ? fused_batch_substage_uxy(b->sw, tile, args, d_items, nitems, d_counters + 3 * p + s, grid, b->stream)
                        : fused_batch_substage_gen(b->sw, tile, args, d_items, nitems, d_counters + 3 * p + s, grid, b->stream);
            if (!rc) rc = fused_batch_bcon(b->sw, args, b->d_bitems, b->nbitems, b->stream);
        }
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
        std::vector<Fused32Args> a32;
        fill_args32(b, cur, a32);
        BCK(cudaMemcpy(b->d_args32, a32.data(), sizeof(Fused32Args) * a32.size(), cudaMemcpyHostToDevice));
    } else {
        std::vector<FusedArgs> args;
        fill_args(b, U0, U1, Z, FT, cur, args);
        BCK(cudaMemcpy(b->d_args, args.data(), sizeof(FusedArgs) * args.size(), cudaMemcpyHostToDevice));
    }
    std::vector<int4> items;
    make_items(b, b->tile, items);
    cudaFree(b->d_items);
    BCK(cudaMalloc(&b->d_items, sizeof(int4) * items.size()));
    BCK(cudaMemcpy(b->d_items, items.data(), sizeof(int4) * items.size(), cudaMemcpyHostToDevice));
    b->nitems = (int)items.size();
    drop_graphs(b->exec);
    int rc = capture(b, b->tile, b->d_args, b->d_items, b->nitems, b->d_counters, b->exec);
    if (rc) return rc;
    b->expect_cur = cur;
    b->phase = 0;
    b->built = true;
    return MHD_OK;
}

// Time every tile shape on a scratch copy of the batch; returns the fastest.
int autotune(mhd_batch* b, double* ms_out) {
    const int n = (int)b->ctx.size();
    std::vector<double*> U0(n), U1(n), Z(n), FT(n);
    std::vector<void*> owned;
    std::vector<int> cur(n, 0);
    int rc = MHD_OK;
    for (int i = 0; i < n && !rc; i++) {
        mhd_ctx* c = b->ctx[i];
        const size_t fb = c->ncell * sizeof(double);
        double* blk = nullptr;
        const int nf_ft = (c->sw & kSwShr) ? 1 : 0;
        if (cudaMalloc(&blk, fb * (24 + nf_ft)) != cudaSuccess) {
            cudaGetLastError();
            rc = bfail(b, MHD_ERR_NOMEM, "autotuner scratch allocation failed");
            break;
        }
        owned.push_back(blk);
        U0[i] = blk;
        U1[i] = blk + 8 * c->ncell;
        Z[i] = blk + 16 * c->ncell;
        FT[i] = nf_ft ? blk + 24 * c->ncell : nullptr;
        cudaMemcpyAsync(U0[i], c->U[c->cur], fb * 8, cudaMemcpyDeviceToDevice, b->stream);
        cudaMemcpyAsync(U1[i], c->U[c->cur], fb * 8, cudaMemcpyDeviceToDevice, b->stream);
        cudaMemsetAsync(Z[i], 0, fb * 8, b->stream);
        if (FT[i]) cudaMemsetAsync(FT[i], 0, fb, b->stream);
    }
    FusedArgs* d_args = nullptr;
    int* d_cnt = nullptr;
    int best = 0;
    double best_ms = 1e300;
    if (!rc && cudaMalloc(&d_args, sizeof(FusedArgs) * 6 * n) != cudaSuccess) rc = MHD_ERR_NOMEM;
    if (!rc && cudaMalloc(&d_cnt, sizeof(int) * 6) != cudaSuccess) rc = MHD_ERR_NOMEM;
    if (!rc) {
        std::vector<FusedArgs> args;
        fill_args(b, U0, U1, Z, FT, cur, args);
        cudaMemcpy(d_args, args.data(), sizeof(FusedArgs) * args.size(), cudaMemcpyHostToDevice);
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        for (int t = 0; t < kBatchTiles && !rc; t++) {
            std::vector<int4> items;
            make_items(b, t, items);
            int4* d_items = nullptr;
            if (cudaMalloc(&d_items, sizeof(int4) * items.size()) != cudaSuccess) {
                rc = MHD_ERR_NOMEM;
                break;
            }
            cudaMemcpy(d_items, items.data(), sizeof(int4) * items.size(), cudaMemcpyHostToDevice);
            cudaGraphExec_t ex[2] = {nullptr, nullptr};
            rc = capture(b, t, d_args, d_items, (int)items.size(), d_cnt, ex);
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
                if (ms_out) ms_out[t] = per;
                if (per < best_ms) {
                    best_ms = per;
                    best = t;
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
        cudaMemcpy(b->d_bitems, bitems.data(), sizeof(int2) * bitems.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
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
    cudaFree(b->d_args);
    cudaFree(b->d_args32);
    cudaFree(b->d_items);
    cudaFree(b->d_bitems);
    cudaFree(b->d_counters);
    if (b->own_stream) cudaStreamDestroy(b->stream);
    delete b;
    return MHD_OK;
}

int mhd_batch_set_tile(mhd_batch* b, int tile) {
    if (!b || tile < -1 || tile >= kBatchTiles) return MHD_ERR_INVALID;
    b->tile = tile;
    b->built = false;
    return MHD_OK;
}

int mhd_batch_autotune(mhd_batch* b, int* chosen, double* ms_per_step) {
    if (!b) return MHD_ERR_INVALID;
    if (b->fp32) {  // one tile shape for FP32 storage: nothing to choose
        b->tile = 0;
        b->built = false;
        if (chosen) *chosen = 0;
        if (ms_per_step)
            for (int t = 0; t < kBatchTiles; t++) ms_per_step[t] = 0.0;
        return MHD_OK;
    }
    const std::string sig = signature(b);
    int best = -1;
    if (!ms_per_step) {
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        auto it = g_tune_cache.find(sig);
        if (it != g_tune_cache.end()) best = it->second;
    }
    if (best < 0) {
        best = autotune(b, ms_per_step);
        if (best < 0) return best;
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        g_tune_cache[sig] = best;
    }
    b->tile = best;
    b->built = false;
    if (chosen) *chosen = best;
    return MHD_OK;
}

int mhd_batch_steps(mhd_batch* b, int nsteps) {
    if (!b || nsteps < 0) return MHD_ERR_INVALID;
    if (b->tile < 0) {
        int rc = mhd_batch_autotune(b, nullptr, nullptr);
        if (rc) return rc;
    }
    bool stale = !b->built;
    for (size_t i = 0; i < b->ctx.size() && !stale; i++)
        stale = b->ctx[i]->cur != b->expect_cur[i] || !b->ctx[i]->ghosts_synced;
    if (stale) {
        int rc = build(b);
        if (rc) return rc;
    }
    if (!b->order) BCK(cudaEventCreateWithFlags(&b->order, cudaEventDisableTiming));
    // work queued on the instances' own streams (uploads, single steps) first
    for (mhd_ctx* c : b->ctx) {
        BCK(cudaEventRecord(b->order, c->stream));
        BCK(cudaStreamWaitEvent(b->stream, b->order, 0));
    }
    for (int s = 0; s < nsteps; s++) {
        BCK(cudaGraphLaunch(b->exec[b->phase], b->stream));
        b->phase ^= 1;
        for (size_t i = 0; i < b->ctx.size(); i++) {
            mhd_ctx* c = b->ctx[i];
            c->cur ^= 1;
            b->expect_cur[i] ^= 1;
            ctxops::advance_time(c, b->dt[i]);
        }
        b->steps_done++;
    }
    // later work on an instance's stream (downloads, diagnostics) waits for the batch
    BCK(cudaEventRecord(b->order, b->stream));
    for (mhd_ctx* c : b->ctx) BCK(cudaStreamWaitEvent(c->stream, b->order, 0));
    return MHD_OK;
}

int mhd_batch_sync(mhd_batch* b) {
    if (!b) return MHD_ERR_INVALID;
    BCK(cudaStreamSynchronize(b->stream));
    return MHD_OK;
}

int mhd_batch_tile(const mhd_batch* b, int* tile) {
    if (!b || !tile) return MHD_ERR_INVALID;
    *tile = b->tile;
    return MHD_OK;
}

}  // extern "C"
