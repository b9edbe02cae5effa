// mhd_pipeline.cu -- fused FP64 steps from a host state to a host state with
// the transfers hidden behind the computation.
//
// A driver that keeps its state in host memory (the reference's arrays) pays
// an upload and a download of the whole state around every step.  Here the
// interior z planes are cut into slabs and the step runs as a dataflow over
// five streams, one per kind of work:
//   copy-in          slab j (all fields) and the first plane of slab j+1 -> U[cur],
//                    then event up[j]
//   substage s=1..3  S_s(j) after up[j] (S1), or after stage s-1 of slab j+1
//                    (S1 done[j+1] for S2, S2 done[j+1] for S3)
//   copy-out         slab j of the new state after S3 done[j]
// Substage s of slab j reads its neighbours one plane beyond the slab, which
// came with the slab's upload (S1) or which stage s-1 of slab j+1 has
// produced by then (S2, S3: waiting for the whole slab j+1 of S1 would hold
// S1 a slab behind the uploads for no reason); the same events order the
// in-place ping-pong writes (S2(j) overwrites U[cur] planes that S1 of slabs
// j-1..j+1 read, S3(j) overwrites U[1-cur] planes that S2 of slabs j-1..j+1
// read), and the substages of one slab follow one another through it.  The
// wall BCON of each substage follows its first / last slab on the same
// stream.  Kernels of different substages run concurrently, so one kernel's
// last wave overlaps the next kernel's first instead of draining the GPU; the
// later substages have the higher stream priority, so the pipeline drains
// early.  Every cell goes through the same arithmetic as in mhd_step, so the
// result is bit-identical to upload + mhd_step + download.
//
// mhd_steps_host chains n such steps without a host synchronisation between
// them: step k+1's upload of slab j waits only for step k's download of slab
// j+1, so the first slabs of one step overlap the last slabs and downloads of
// the step before instead of waiting for them to drain.
#include "mhd_context.h"

#include <algorithm>
#include <vector>

namespace {

using namespace mhd;

int fail_cuda(mhd_ctx* c, cudaError_t e, const char* where) {
    return ctxops::fail(c, MHD_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define PCK(call)                                                \
    do {                                                         \
        cudaError_t e_ = (call);                                 \
        if (e_ != cudaSuccess) return fail_cuda(ctx, e_, #call); \
    } while (0)

// copy planes [z0, z1) of every state field between host (field-major,
// nf x nz x ny x nx) and device buffer `dev`
cudaError_t copy_planes(const mhd_ctx* ctx, double* dev, double* host, int z0, int z1, bool up, cudaStream_t st) {
    const size_t plane = (size_t)ctx->g.sz, off = (size_t)z0 * plane, n = (size_t)(z1 - z0) * plane;
    for (int f = 0; f < ctx->nf; f++) {
        double* d = dev + (size_t)f * ctx->ncell + off;
        double* h = host + (size_t)f * ctx->ncell + off;
        cudaError_t e = up ? cudaMemcpyAsync(d, h, n * sizeof(double), cudaMemcpyHostToDevice, st)
                           : cudaMemcpyAsync(h, d, n * sizeof(double), cudaMemcpyDeviceToHost, st);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// Interior slab bounds: heights grow geometrically from the bottom wall, 4,
// 4, 8, 16, then about 32 planes, and shrink again, 24, 16, 12, 8, 4 (16, 8,
// 4 below 128 planes), at the top: the compute waits for the first slab's
// upload, each later upload must fit under the compute of the slabs before
// it, and the downloads of the last slabs, which queue behind one another
// after the last kernels, are short.  Every slab has at least 4 planes (the
// wall stencils reach 3 planes in).  Fewer than 3 slabs: no pipeline.
std::vector<int> slab_bounds(int nPz) {
    std::vector<int> b{1};
    const int head[4] = {4, 4, 8, 16}, tail_long[5] = {24, 16, 12, 8, 4}, tail_short[3] = {16, 8, 4};
    if (nPz >= 92) {
        const bool lt = nPz >= 32 + 64 + 32;
        const int* tail = lt ? tail_long : tail_short;
        const int nt = lt ? 5 : 3, st = lt ? 64 : 28;
        for (int h : head) b.push_back(b.back() + h);
        const int mid = nPz - 32 - st, nm = std::max(1, (mid + 16) / 32), m0 = b.back();
        for (int j = 1; j <= nm; j++) b.push_back(m0 + (int)((long long)mid * j / nm));
        for (int t = 0; t < nt; t++) b.push_back(b.back() + tail[t]);
    }
    return b;
}

// Streams and events of the pipeline, created on first use.
int ensure_pipeline(mhd_ctx* ctx, int ns) {
    if (!ctx->s_up) {
        int lo = 0, hi = 0;
        PCK(cudaDeviceGetStreamPriorityRange(&lo, &hi));  // hi: numerically smallest, most urgent
        PCK(cudaStreamCreateWithFlags(&ctx->s_up, cudaStreamNonBlocking));
        PCK(cudaStreamCreateWithFlags(&ctx->s_down, cudaStreamNonBlocking));
        for (int s = 0; s < 3; s++) {
            const int pr = lo + (hi - lo) * s / 2;  // S1 least urgent, S3 most
            PCK(cudaStreamCreateWithPriority(&ctx->s_sub[s], cudaStreamNonBlocking, pr));
        }
    }
    const size_t need = 5 * (size_t)ns + 2;
    while (ctx->slab_events.size() < need) {
        cudaEvent_t e;
        PCK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        ctx->slab_events.push_back(e);
    }
    return MHD_OK;
}

// Enqueue one step on the pipeline streams (no host synchronisation).
// `chained`: the previous step was enqueued by this function and nothing ran
// on the context's stream since; then this step starts without a barrier:
// its upload of slab j waits for the previous step's download of slab j+1
// (`prev_out`: the previous step downloaded), else its substage 1 of slab j
// waits for the previous step's substage 3 of slab j+1.  Either orders every
// write of this step after the previous step's reads of the same planes (that
// step's substage 3 of slabs <= j+1 and its downloads of slabs <= j+1 are then
// done), and the upload after the download of the same host planes.
int issue_step(mhd_ctx* ctx, const std::vector<int>& b, const double* in, double* out, double dt, bool chained,
               bool prev_out) {
    const int ns = (int)b.size() - 1, nz = ctx->g.nz;
    int rc = ctxops::plume_update(ctx, ctx->timt);
    if (rc) return rc;
    // ev[0] = up[ns], ev[1..3] = done of substage 1..3 [ns], ev[4] = down[ns]
    cudaEvent_t* ev[5];
    for (int k = 0; k < 5; k++) ev[k] = ctx->slab_events.data() + (size_t)k * ns;
    cudaEvent_t start = ctx->slab_events[5 * (size_t)ns];
    auto lo_of = [&](int j) { return j == 0 ? 0 : b[j]; };  // with the ghost planes
    auto hi_of = [&](int j) { return j == ns - 1 ? nz : b[j + 1]; };
    auto next = [&](int j) { return std::min(j + 1, ns - 1); };

    const int cur = ctx->cur;
    double* Uin = ctx->U[cur];
    double* Uout = ctx->U[1 - cur];  // after three substages the state is in U[1-cur]
    if (!chained) {
        if (!in) {
            int r2 = ctxops::sync_zghosts(ctx);
            if (r2) return r2;
        }
        // every stream starts after everything queued on the context's stream
        PCK(cudaEventRecord(start, ctx->stream));
        PCK(cudaStreamWaitEvent(ctx->s_up, start, 0));
        PCK(cudaStreamWaitEvent(ctx->s_down, start, 0));
        for (int s = 0; s < 3; s++) PCK(cudaStreamWaitEvent(ctx->s_sub[s], start, 0));
    }
    ctx->ghosts_synced = true;
    // up[j]: slab j and the first plane of slab j+1, all that S1 of slab j reads
    auto up_hi = [&](int j) { return j == ns - 1 ? nz : hi_of(j) + 1; };
    for (int j = 0; j < ns; j++) {
        if (in) {
            if (chained && prev_out) PCK(cudaStreamWaitEvent(ctx->s_up, ev[4][next(j)], 0));
            PCK(copy_planes(ctx, Uin, const_cast<double*>(in), j == 0 ? 0 : up_hi(j - 1), up_hi(j), true, ctx->s_up));
            // the z ghost planes are never written by a substage: both buffers hold them
            if (j == 0) PCK(copy_planes(ctx, Uout, const_cast<double*>(in), 0, 1, true, ctx->s_up));
            if (j == ns - 1) PCK(copy_planes(ctx, Uout, const_cast<double*>(in), nz - 1, nz, true, ctx->s_up));
        }
        PCK(cudaEventRecord(ev[0][j], ctx->s_up));
    }

    auto substage = [&](int s, int j) -> int {
        cudaStream_t st = ctx->s_sub[s];
        FusedArgs a = ctxops::fused_args(ctx, s, dt, s == 1 ? 1 - cur : cur);
        a.zlo = b[j];
        a.zhi = b[j + 1];
        int e = fused_substage(ctx->sw, a, st);
        if (e) return fail_cuda(ctx, (cudaError_t)e, "fused substage launch");
        if (j == 0) e = fused_bcon_wall(ctx->sw, ctx->g, ctx->c, a.Uo, ctx->timt, 0, st);
        if (!e && j == ns - 1) e = fused_bcon_wall(ctx->sw, ctx->g, ctx->c, a.Uo, ctx->timt, 1, st);
        if (e) return fail_cuda(ctx, (cudaError_t)e, "BCON launch");
        return MHD_OK;
    };
    // issue in wavefront order (S1 of slab t, S2 of t-1, S3 of t-2), so each
    // wait names an event that is already recorded; the previous step's
    // substage-3 events a chained S1 waits for (slabs t+1) are re-recorded by
    // this step only at wavefront t+3
    for (int t = 0; t < ns + 2; t++) {
        for (int s = 0; s < 3; s++) {
            const int j = t - s;
            if (j < 0 || j >= ns) continue;
            if (s == 0 && chained && !(in && prev_out)) PCK(cudaStreamWaitEvent(ctx->s_sub[0], ev[3][next(j)], 0));
            PCK(cudaStreamWaitEvent(ctx->s_sub[s], ev[s][s == 0 ? j : next(j)], 0));
            if ((rc = substage(s, j))) return rc;
            PCK(cudaEventRecord(ev[s + 1][j], ctx->s_sub[s]));
            if (s == 2 && out) {
                PCK(cudaStreamWaitEvent(ctx->s_down, ev[3][j], 0));
                PCK(copy_planes(ctx, Uout, out, lo_of(j), hi_of(j), false, ctx->s_down));
                PCK(cudaEventRecord(ev[4][j], ctx->s_down));
            }
        }
    }
    ctx->cur = 1 - cur;
    ctxops::advance_time(ctx, dt);
    return MHD_OK;
}

// After the last enqueued step: later work on the context's stream waits for
// the last download (or the last substage-3 kernel), which follow every other
// operation of the steps; blocks when there were downloads.
int finish_steps(mhd_ctx* ctx, int ns, bool downloaded) {
    cudaEvent_t fin = ctx->slab_events[5 * (size_t)ns + 1];
    PCK(cudaEventRecord(fin, downloaded ? ctx->s_down : ctx->s_sub[2]));
    PCK(cudaStreamWaitEvent(ctx->stream, fin, 0));
    if (downloaded) PCK(cudaStreamSynchronize(ctx->stream));
    return MHD_OK;
}

// Checks and set-up shared by both entry points; *ns = 0: the plain path.
int prepare(mhd_ctx* ctx, double dt, std::vector<int>& b) {
    if (!ctx || !(dt > 0.0)) return MHD_ERR_INVALID;
    if (ctx->fp32 || ctx->prm.path != MHD_PATH_FUSED)
        return ctxops::fail(ctx, MHD_ERR_UNSUPPORTED, "host-to-host steps run on the fused FP64 path");
    b = slab_bounds(ctx->g.nz - 2);
    const int ns = (int)b.size() - 1;
    if (ns < 3 || ctx->c.lrem) {
        // too thin to pipeline (or lRem, whose substages need whole-plane
        // means first): upload, step, download
        b.clear();
        return MHD_OK;
    }
    int rc = ctxops::ensure_u1(ctx);
    if (!rc && (ctx->sw & kSwShr)) rc = ctxops::alloc_block(ctx, &ctx->Fb, 8);
    if (!rc) rc = ensure_pipeline(ctx, ns);
    return rc;
}

int plain_step(mhd_ctx* ctx, const double* in, double* out, double dt) {
    int rc = in ? mhd_upload_state(ctx, in) : MHD_OK;
    if (!rc) rc = mhd_step(ctx, dt, nullptr);
    if (!rc && out) rc = mhd_download_state(ctx, out);
    return rc;
}

}  // namespace

extern "C" int mhd_step_host(mhd_ctx* ctx, const double* in, double* out, double dt) {
    std::vector<int> b;
    int rc = prepare(ctx, dt, b);
    if (rc) return rc;
    if (b.empty()) return plain_step(ctx, in, out, dt);
    rc = issue_step(ctx, b, in, out, dt, false, false);
    if (rc) return rc;
    return finish_steps(ctx, (int)b.size() - 1, out != nullptr);
}

extern "C" int mhd_steps_host(mhd_ctx* ctx, int n, const double* in, double* out, double dt) {
    if (n < 0) return MHD_ERR_INVALID;
    std::vector<int> b;
    int rc = prepare(ctx, dt, b);
    if (rc || n == 0) return rc;
    for (int k = 0; k < n; k++) {
        // step 0 reads `in`, every later step the previous result in `out`
        const double* src = k == 0 ? in : out;
        if (b.empty()) rc = plain_step(ctx, src, out, dt);
        else rc = issue_step(ctx, b, src, out, dt, k > 0, out != nullptr);
        if (rc) return rc;
    }
    if (b.empty()) return MHD_OK;
    return finish_steps(ctx, (int)b.size() - 1, out != nullptr);
}
