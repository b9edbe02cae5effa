// mhd_pipeline.cu -- one fused FP64 step from a host state to a host state
// with the transfers hidden behind the computation.
//
// A driver that keeps its state in host memory (the reference's arrays) pays
// an upload and a download of the whole state around every step.  Here the
// interior z planes are cut into slabs and the step runs as a wavefront over
// three streams:
//   copy-in stream   slab j (all fields) -> U[cur], then event up[j]
//   compute stream   S1(t) after up[t+1];  S2(t-1);  S3(t-2), then event done[t-2]
//   copy-out stream  slab j of the new state after done[j]
// Substage s of slab j reads its neighbours one plane beyond the slab, which
// substage s-1 has finished by then (slab j+1 was issued earlier on the same
// stream); the wall BCON of each substage follows the first / last slab.  The
// in-place reads and writes of the ping-pong buffers are ordered by the issue
// order: S1(j+1) is issued before S2(j) overwrites the plane it reads, and
// S2(j+1) before S3(j).  Every cell goes through the same arithmetic as in
// mhd_step, so the result is bit-identical to upload + mhd_step + download.
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

}  // namespace

extern "C" int mhd_step_host(mhd_ctx* ctx, const double* in, double* out, double dt) {
    if (!ctx || !(dt > 0.0)) return MHD_ERR_INVALID;
    if (ctx->fp32 || ctx->prm.path != MHD_PATH_FUSED)
        return ctxops::fail(ctx, MHD_ERR_UNSUPPORTED, "host-to-host steps run on the fused FP64 path");
    const int nPz = ctx->g.nz - 2, nz = ctx->g.nz;
    // Interior slab heights grow geometrically from the bottom wall, 4, 4, 8,
    // 16, then about 32 planes, and shrink again, 16, 8, 4, at the top: the
    // compute waits for the first two slabs' upload, each later upload must
    // fit under the compute of the slabs before it (a plane uploads in about
    // 0.7x the time its three substages take at 512 x 512), and the last
    // download follows the last kernel.  Every slab has at least 4 planes (the
    // wall stencils reach 3 planes in).
    std::vector<int> b{1};
    const int head[4] = {4, 4, 8, 16}, tail[3] = {16, 8, 4};
    if (nPz >= 92) {
        for (int h : head) b.push_back(b.back() + h);
        const int mid = nPz - 32 - 28, nm = std::max(1, (mid + 16) / 32), m0 = b.back();
        for (int j = 1; j <= nm; j++) b.push_back(m0 + (int)((long long)mid * j / nm));
        for (int h : tail) b.push_back(b.back() + h);
    }
    const int ns = (int)b.size() - 1;
    if (ns < 3 || ctx->c.lrem) {
        // too thin to pipeline (or lRem, whose substages need whole-plane
        // means first): upload, step, download
        int rc = in ? mhd_upload_state(ctx, in) : MHD_OK;
        if (!rc) rc = mhd_step(ctx, dt, nullptr);
        if (!rc && out) rc = mhd_download_state(ctx, out);
        return rc;
    }
    int rc = ctxops::ensure_u1(ctx);
    if (!rc && (ctx->sw & kSwShr)) rc = ctxops::alloc_block(ctx, &ctx->Fb, 8);
    if (!rc) rc = ctxops::plume_update(ctx, ctx->timt);
    if (rc) return rc;
    if (!ctx->s_up) {
        PCK(cudaStreamCreateWithFlags(&ctx->s_up, cudaStreamNonBlocking));
        PCK(cudaStreamCreateWithFlags(&ctx->s_down, cudaStreamNonBlocking));
    }
    const size_t need = 2 * (size_t)ns + 2;
    while (ctx->slab_events.size() < need) {
        cudaEvent_t e;
        PCK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        ctx->slab_events.push_back(e);
    }
    cudaEvent_t* up = ctx->slab_events.data();          // [ns]
    cudaEvent_t* done = up + ns;                        // [ns]
    cudaEvent_t start = done[ns], fin = done[ns + 1];
    auto lo_of = [&](int j) { return j == 0 ? 0 : b[j]; };       // with the ghost planes
    auto hi_of = [&](int j) { return j == ns - 1 ? nz : b[j + 1]; };

    const int cur = ctx->cur;
    double* Uin = ctx->U[cur];
    double* Uout = ctx->U[1 - cur];  // after three substages the state is in U[1-cur]
    // the copy streams start after everything queued on the context's stream
    PCK(cudaEventRecord(start, ctx->stream));
    PCK(cudaStreamWaitEvent(ctx->s_up, start, 0));
    PCK(cudaStreamWaitEvent(ctx->s_down, start, 0));
    for (int j = 0; j < ns; j++) {
        if (in) {
            PCK(copy_planes(ctx, Uin, const_cast<double*>(in), lo_of(j), hi_of(j), true, ctx->s_up));
            // the z ghost planes are never written by a substage: both buffers hold them
            if (j == 0) PCK(copy_planes(ctx, Uout, const_cast<double*>(in), 0, 1, true, ctx->s_up));
            if (j == ns - 1) PCK(copy_planes(ctx, Uout, const_cast<double*>(in), nz - 1, nz, true, ctx->s_up));
        }
        PCK(cudaEventRecord(up[j], ctx->s_up));
    }
    if (!in) {
        int r2 = ctxops::sync_zghosts(ctx);
        if (r2) return r2;
    }
    ctx->ghosts_synced = true;

    auto substage = [&](int s, int j) -> int {
        FusedArgs a = ctxops::fused_args(ctx, s, dt, s == 1 ? 1 - cur : cur);
        a.zlo = b[j];
        a.zhi = b[j + 1];
        int e = fused_substage(ctx->sw, a, ctx->stream);
        if (e) return fail_cuda(ctx, (cudaError_t)e, "fused substage launch");
        if (j == 0) e = fused_bcon_wall(ctx->sw, ctx->g, ctx->c, a.Uo, ctx->timt, 0, ctx->stream);
        if (!e && j == ns - 1) e = fused_bcon_wall(ctx->sw, ctx->g, ctx->c, a.Uo, ctx->timt, 1, ctx->stream);
        if (e) return fail_cuda(ctx, (cudaError_t)e, "BCON launch");
        return MHD_OK;
    };
    for (int t = 0; t < ns + 2; t++) {
        if (t < ns) {
            PCK(cudaStreamWaitEvent(ctx->stream, up[std::min(t + 1, ns - 1)], 0));
            if ((rc = substage(0, t))) return rc;
        }
        if (t - 1 >= 0 && t - 1 < ns && (rc = substage(1, t - 1))) return rc;
        if (t - 2 >= 0 && t - 2 < ns) {
            const int j = t - 2;
            if ((rc = substage(2, j))) return rc;
            PCK(cudaEventRecord(done[j], ctx->stream));
            if (out) {
                PCK(cudaStreamWaitEvent(ctx->s_down, done[j], 0));
                PCK(copy_planes(ctx, Uout, out, lo_of(j), hi_of(j), false, ctx->s_down));
            }
        }
    }
    // later work on the context's stream waits for the copies
    PCK(cudaEventRecord(fin, ctx->s_down));
    PCK(cudaStreamWaitEvent(ctx->stream, fin, 0));
    ctx->cur = 1 - cur;
    ctxops::advance_time(ctx, dt);
    if (out) PCK(cudaStreamSynchronize(ctx->stream));
    return MHD_OK;
}
