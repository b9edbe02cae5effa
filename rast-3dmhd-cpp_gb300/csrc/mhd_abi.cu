// mhd_abi.cu -- host side of the C ABI declared in include/mhd_gb300.h.
//
// A context replaces the reference's static globals (3dmhd.cpp:29-39) by
// device buffers:
//   U[2]   two copies of the state (RU RV RW TT RO BX BY BZ), ping-ponged by
//          the fused path, each field a full [nz][ny][nx] array with ghosts
//   Z      the RK register (ZRU ... ZBZ)
//   F      the right-hand sides (FU FV FW FR FT WW1 WW2 WW3); the fused path
//          only keeps FT, and only with lShr (where the reference carries it
//          across substages)
//   S      scratch of the unfused path: p = rho*T and the velocities
// Buffers that a call sequence never needs are allocated on first use.
#include "mhd_context.h"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

using namespace mhd;




namespace {

int fail(mhd_ctx* c, int code, const std::string& msg) {
    if (c) c->err = msg;
    return code;
}

int cuda_fail(mhd_ctx* c, cudaError_t e, const char* where) {
    return fail(c, MHD_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define CK(call)                                                \
    do {                                                        \
        cudaError_t e_ = (call);                                \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call); \
    } while (0)

size_t field_bytes(const mhd_ctx* c) { return c->ncell * sizeof(double); }

int alloc_block(mhd_ctx* ctx, double** p, int nfields) {
    if (*p) return MHD_OK;
    const size_t b = field_bytes(ctx) * (size_t)nfields;
    cudaError_t e = cudaMalloc(p, b);
    if (e != cudaSuccess) {
        *p = nullptr;
        cudaGetLastError();
        return fail(ctx, MHD_ERR_NOMEM, "device allocation of " + std::to_string(b) + " bytes failed");
    }
    ctx->bytes += b;
    e = cudaMemsetAsync(*p, 0, b, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMemsetAsync");
    return MHD_OK;
}

Fields8 fields_of(const mhd_ctx* c, double* base) {
    Fields8 f{};
    for (int k = 0; k < 8; k++) f.p[k] = base ? base + (size_t)k * c->ncell : nullptr;
    return f;
}

// Derived scalars exactly as set() and main() compute them: the literals of
// 3dmhd.cpp:354-369 are single precision; 3dmhd.cpp:432-438,451-459; 144-145.
void compute_constants(const mhd_params& p, mhd_constants& k) {
    k.C13 = 1.0f / 3.0f;
    k.C23 = 2.0f * k.C13;
    k.C43 = 4.0f * k.C13;
    k.GAM1 = 8.0f / 15.0f;
    k.GAM2 = 5.0f / 12.0f;
    k.GAM3 = 3.0f / 4.0f;
    k.ZETA1 = -17.0f / 60.0f;
    k.ZETA2 = -5.0f / 12.0f;
    k.hx = 0.5f * float(p.nPx - 1);
    k.h2x = float(p.nPx - 1) * float(p.nPx - 1);
    k.hy = 0.5f * float(p.nPy - 1);
    k.h2y = float(p.nPy - 1) * float(p.nPy - 1);
    k.hz = 0.5f * float(p.nPz - 1);
    k.h2z = float(p.nPz - 1) * float(p.nPz - 1);
    if (p.switches & MHD_SW_LROT) {
        k.OMX = std::sin(p.ANG) / p.RY;
        k.OMZ = std::cos(p.ANG) / p.RY;
    } else {
        k.OMX = 0.0f;
        k.OMZ = 0.0f;
    }
    k.REPR = p.RE * p.PR;
    k.ORE = 1.0f / p.RE;
    k.ORM = 1.0f / p.RM;
    k.OBETA = 2.0f / p.BETA;
    k.CV = 1.0f / (p.GAMMA - 1.0f);
    k.OCV = 1.0f / k.CV;
}

int validate(const mhd_params* p, std::string& why) {
    if (!p) return why = "params is NULL", MHD_ERR_INVALID;
    if (p->nPx < 2 || p->nPy < 2) return why = "nPx and nPy must be >= 2", MHD_ERR_INVALID;
    if (p->nPz < 4) return why = "nPz must be >= 4 (one-sided wall stencils reach 4 planes)", MHD_ERR_INVALID;
    const double cells = (double)(p->nPx + 2) * (p->nPy + 2) * (p->nPz + 2);
    if (cells > 2.0e9) return why = "grid too large for 32-bit plane indexing", MHD_ERR_INVALID;
    if (p->ixCon != 0 || p->iyCon != 0) return why = "only periodic horizontal boundaries (ixCon=iyCon=0) exist in the reference", MHD_ERR_UNSUPPORTED;
    if ((p->switches & MHD_SW_LREM) && (p->switches & MHD_SW_LSHR))
        return why = "lRem with lShr: the reference's temperature terms then read arrays it did not fill this call (3dmhdsub.h:292-313)",
               MHD_ERR_UNSUPPORTED;
    if (p->izCon != 0 && p->izCon != 1) return why = "izCon must be 0 or 1", MHD_ERR_UNSUPPORTED;
    if (p->iTCon != 0 && p->iTCon != 1 && p->iTCon != 2 && p->iTCon != 4)
        return why = "iTCon must be 0, 1, 2 or 4", MHD_ERR_UNSUPPORTED;
    if (p->iBCon != 0) return why = "iBCon must be 0", MHD_ERR_UNSUPPORTED;
    if (p->precision != MHD_PREC_FP64 && p->precision != MHD_PREC_FP32) return why = "unknown precision", MHD_ERR_INVALID;
    if (p->precision == MHD_PREC_FP32 && p->path != MHD_PATH_FUSED)
        return why = "FP32 storage exists only on the fused path", MHD_ERR_UNSUPPORTED;
    if (p->path != MHD_PATH_FUSED && p->path != MHD_PATH_PARITY) return why = "unknown kernel path", MHD_ERR_INVALID;
    if (!(p->RE > 0) || !(p->RM > 0) || !(p->BETA > 0) || !(p->PR > 0) || !(p->GAMMA > 1))
        return why = "RE, RM, BETA, PR must be > 0 and GAMMA > 1", MHD_ERR_INVALID;
    const double* arrs[11] = {p->dxxdx, p->d2xxdx2, p->DDX, p->dyydy, p->d2yydy2, p->DDY,
                              p->dzzdz, p->d2zzdz2, p->DDZ, p->RKAPA, p->DKAPA};
    for (int i = 0; i < 11; i++)
        if (!arrs[i]) return why = "a metric array pointer is NULL", MHD_ERR_INVALID;
    return MHD_OK;
}

int ensure_u1(mhd_ctx* ctx) {
    if (!ctx->U[1]) {
        int rc = alloc_block(ctx, &ctx->U[1], 8);
        if (rc) return rc;
        ctx->ghosts_synced = false;
    }
    return MHD_OK;
}

// The fused path writes every cell of U[1-cur] except the z ghost planes:
// copy those from U[cur] when they may differ.
int sync_zghosts(mhd_ctx* ctx) {
    if (ctx->ghosts_synced) return MHD_OK;
    const size_t plane = (size_t)ctx->g.sz * sizeof(double);
    double* a = ctx->U[ctx->cur];
    double* b = ctx->U[1 - ctx->cur];
    for (int f = 0; f < 8; f++) {
        double* fa = a + (size_t)f * ctx->ncell;
        double* fb = b + (size_t)f * ctx->ncell;
        CK(cudaMemcpyAsync(fb, fa, plane, cudaMemcpyDeviceToDevice, ctx->stream));
        const size_t last = (size_t)(ctx->g.nz - 1) * ctx->g.sz;
        CK(cudaMemcpyAsync(fb + last, fa + last, plane, cudaMemcpyDeviceToDevice, ctx->stream));
    }
    ctx->ghosts_synced = true;
    return MHD_OK;
}

int ensure_parity_buffers(mhd_ctx* ctx) {
    int rc = alloc_block(ctx, &ctx->Fb, 8);
    if (rc) return rc;
    return alloc_block(ctx, &ctx->Sb, 4);
}

// One fused FP64 step; dtp (device) = the time-step record of mhd_steps_cfl,
// from which the kernels read dt, or null for the host dt.
int fused_step(mhd_ctx* ctx, double dt, const double* dtp = nullptr) {
    int rc = ensure_u1(ctx);
    if (rc) return rc;
    if (ctx->sw & kSwShr) {
        rc = alloc_block(ctx, &ctx->Fb, 8);
        if (rc) return rc;
    }
    rc = sync_zghosts(ctx);
    if (rc) return rc;
    for (int s = 0; s < 3; s++) {
        FusedArgs a = ctxops::fused_args(ctx, s, dt, ctx->cur);
        a.dtp = dtp;
        if (ctx->c.lrem) {
            // horizontal means of the substage's input T (3dmhdsub.h:297-313)
            const int e = lrem_profiles(ctx->g, ctx->c, a.U.p[S_TT], ctx->d_lrem, false, ctx->stream);
            if (e) return cuda_fail(ctx, (cudaError_t)e, "lRem profiles launch");
        }
        cudaEvent_t* ev = nullptr;
        if (ctx->profiling) {
            if (ctx->prof_used + 2 > ctx->prof_events.size()) {
                for (int j = 0; j < 64; j++) {
                    cudaEvent_t e0;
                    CK(cudaEventCreate(&e0));
                    ctx->prof_events.push_back(e0);
                }
            }
            ev = &ctx->prof_events[ctx->prof_used];
            ctx->prof_used += 2;
            CK(cudaEventRecord(ev[0], ctx->stream));
        }
        int e = fused_substage(ctx->sw, a, ctx->stream);
        if (e) return cuda_fail(ctx, (cudaError_t)e, "fused substage launch");
        if (ev) CK(cudaEventRecord(ev[1], ctx->stream));
        e = fused_bcon_ghost(ctx->sw, ctx->g, ctx->c, a.Uo, ctx->timt, ctx->stream);
        if (e) return cuda_fail(ctx, (cudaError_t)e, "BCON launch");
        ctx->cur = 1 - ctx->cur;
    }
    return MHD_OK;
}

int alloc_f32(mhd_ctx* ctx, float** p) {
    if (*p) return MHD_OK;
    const size_t b = ctx->ncell * sizeof(float) * 8;
    cudaError_t e = cudaMalloc(p, b);
    if (e != cudaSuccess) {
        *p = nullptr;
        cudaGetLastError();
        return fail(ctx, MHD_ERR_NOMEM, "device allocation of " + std::to_string(b) + " bytes failed");
    }
    ctx->bytes += b;
    e = cudaMemsetAsync(*p, 0, b, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMemsetAsync");
    return MHD_OK;
}

Fields8f fields32_of(const mhd_ctx* c, float* base) {
    Fields8f f{};
    for (int k = 0; k < 8; k++) f.p[k] = base ? base + (size_t)k * c->ncell : nullptr;
    return f;
}

// Profile of a state field in the FP32 layout: RO -> rho0, TT -> T0, others none.
const double* profile_host(const mhd_ctx* c, int field) {
    const int nz = c->g.nz;
    if (field == MHD_RO) return c->h_bg.data();
    if (field == MHD_TT) return c->h_bg.data() + nz;
    return nullptr;
}

// rho0 / T0 := horizontal mean of the uploaded field over interior (y, x), per z;
// for T0 also its premultiplied first and second z derivatives.
int set_profile(mhd_ctx* ctx, int field, const double* host) {
    const int nx = ctx->g.nx, ny = ctx->g.ny, nz = ctx->g.nz;
    double* bg = ctx->h_bg.data() + (field == MHD_RO ? 0 : nz);
    for (int z = 0; z < nz; z++) {
        double s = 0.0;
        for (int y = 1; y < ny - 1; y++)
            for (int x = 1; x < nx - 1; x++) s += host[((size_t)z * ny + y) * nx + x];
        bg[z] = s / ((double)(nx - 2) * (ny - 2));
    }
    return ctxops::profiles_from_means(ctx);
}

}  // namespace

namespace mhd::ctxops {
// With rho0 and T0 in h_bg: T0's premultiplied z derivatives, the float
// coefficient table, and both uploaded.
int profiles_from_means(mhd_ctx* ctx) {
    const int nz = ctx->g.nz;
    const double* bg = ctx->h_bg.data() + nz;
    {
        double* d1 = ctx->h_bg.data() + 2 * nz;
        double* d2 = ctx->h_bg.data() + 3 * nz;
        const double *cz1 = ctx->h_cz.data(), *cz2a = cz1 + nz, *cz2b = cz1 + 2 * nz;
        for (int z = 0; z < nz; z++) {
            d1[z] = d2[z] = 0.0;
            if (z == 0 || z == nz - 1) continue;
            const double p = bg[z + 1], m = bg[z - 1];
            d1[z] = (p - m) * cz1[z];
            d2[z] = (p - m) * cz2a[z] + (p + m - 2.0 * bg[z]) * cz2b[z];
        }
    }
    // the profiles' hydrostatic residual rho0 GRAV - D_z(rho0 T0) per interior z, in
    // FP64 (the two terms nearly cancel); the FP32 kernels add the deviations to it
    const double* r0 = ctx->h_bg.data();
    const double* cz1 = ctx->h_cz.data();
    for (int z = 0; z < nz; z++) {
        ctx->h_zf[3 * (size_t)nz + z] = (float)ctx->h_bg[2 * (size_t)nz + z];
        ctx->h_zf[4 * (size_t)nz + z] = (float)ctx->h_bg[3 * (size_t)nz + z];
        double hz = 0.0;
        if (z > 0 && z < nz - 1) hz = r0[z] * ctx->prm.GRAV - (r0[z + 1] * bg[z + 1] - r0[z - 1] * bg[z - 1]) * cz1[z];
        ctx->h_zf[7 * (size_t)nz + z] = (float)hz;
        // rho0 and T0 as float pairs hi + lo (hi the nearest float, lo the
        // nearest float to the exact remainder): about 48 significant bits,
        // for the FP32 kernels' compensated reconstruction of rho and p
        const float rh = (float)r0[z], th = (float)bg[z];
        ctx->h_zf[8 * (size_t)nz + z] = rh;
        ctx->h_zf[9 * (size_t)nz + z] = (float)(r0[z] - (double)rh);
        ctx->h_zf[10 * (size_t)nz + z] = th;
        ctx->h_zf[11 * (size_t)nz + z] = (float)(bg[z] - (double)th);
    }
    // on the context's stream: its kernels read the profiles (a plain cudaMemcpy
    // runs on the legacy stream, which the non-blocking context stream does not
    // wait for); the sync keeps h_bg / h_zf stable until the copies are done
    CK(cudaMemcpyAsync(ctx->d_bg, ctx->h_bg.data(), sizeof(double) * 4 * nz, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->d_bg + 4 * nz, ctx->h_zf.data(), sizeof(float) * kZfRows * nz, cudaMemcpyHostToDevice,
                       ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return MHD_OK;
}
}  // namespace mhd::ctxops

namespace {

int upload32(mhd_ctx* ctx, int field, const double* host) {
    if (field == MHD_RO || field == MHD_TT) {
        int rc = set_profile(ctx, field, host);
        if (rc) return rc;
    }
    const double* bg = profile_host(ctx, field);
    const size_t plane = (size_t)ctx->g.sz;
    std::vector<float> tmp(ctx->ncell);
    for (size_t i = 0; i < ctx->ncell; i++) tmp[i] = (float)(host[i] - (bg ? bg[i / plane] : 0.0));
    CK(cudaMemcpyAsync(ctx->U32[ctx->cur] + (size_t)field * ctx->ncell, tmp.data(), ctx->ncell * sizeof(float),
                       cudaMemcpyHostToDevice, ctx->stream));
    // the FP64 register carries the full state between steps
    CK(cudaMemcpyAsync(ctx->Zb + (size_t)field * ctx->ncell, host, ctx->ncell * sizeof(double), cudaMemcpyHostToDevice,
                       ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));  // tmp and the caller's array may go away after return
    ctx->ghosts_synced = false;
    return MHD_OK;
}

int download32(mhd_ctx* ctx, int field, double* host) {
    std::vector<float> tmp(ctx->ncell);
    CK(cudaStreamSynchronize(ctx->stream));
    CK(cudaMemcpy(tmp.data(), ctx->U32[ctx->cur] + (size_t)field * ctx->ncell, ctx->ncell * sizeof(float),
                  cudaMemcpyDeviceToHost));
    const double* bg = profile_host(ctx, field);
    const size_t plane = (size_t)ctx->g.sz;
    for (size_t i = 0; i < ctx->ncell; i++) host[i] = (double)tmp[i] + (bg ? bg[i / plane] : 0.0);
    return MHD_OK;
}

int sync_zghosts32(mhd_ctx* ctx) {
    if (ctx->ghosts_synced) return MHD_OK;
    const size_t plane = (size_t)ctx->g.sz * sizeof(float);
    float* a = ctx->U32[ctx->cur];
    float* b = ctx->U32[1 - ctx->cur];
    const size_t last = (size_t)(ctx->g.nz - 1) * ctx->g.sz;
    for (int f = 0; f < 8; f++) {
        float* fa = a + (size_t)f * ctx->ncell;
        float* fb = b + (size_t)f * ctx->ncell;
        CK(cudaMemcpyAsync(fb, fa, plane, cudaMemcpyDeviceToDevice, ctx->stream));
        CK(cudaMemcpyAsync(fb + last, fa + last, plane, cudaMemcpyDeviceToDevice, ctx->stream));
    }
    ctx->ghosts_synced = true;
    return MHD_OK;
}

// One FP32-storage step; dtp as for fused_step.
int fused32_step(mhd_ctx* ctx, double dt, const double* dtp = nullptr) {
    int rc = alloc_f32(ctx, &ctx->U32[1]);
    if (rc) return rc;
    if ((ctx->sw & kSwShr) && !ctx->FT64) {
        rc = alloc_block(ctx, &ctx->FT64, 1);
        if (rc) return rc;
    }
    rc = sync_zghosts32(ctx);
    if (rc) return rc;
    const int nz = ctx->g.nz;
    const double gam[3] = {ctx->k.GAM1, ctx->k.GAM2, ctx->k.GAM3};
    const double zet[3] = {ctx->k.ZETA1, ctx->k.ZETA2, 0.0};
    for (int s = 0; s < 3; s++) {
        Fused32Args a{};
        a.g = ctx->g;
        a.c = ctx->c;
        a.k = ctx->coef;
        a.U = fields32_of(ctx, ctx->U32[ctx->cur]);
        a.Uo = fields32_of(ctx, ctx->U32[1 - ctx->cur]);
        a.Z = fields_of(ctx, ctx->Zb);
        a.FT = ctx->FT64;
        a.bgR = ctx->d_bg;
        a.bgT = ctx->d_bg + nz;
        a.dzT0 = ctx->d_bg + 2 * nz;
        a.d2zT0 = ctx->d_bg + 3 * nz;
        a.zf = reinterpret_cast<const float*>(ctx->d_bg + 4 * nz);
        a.gdt = gam[s] * dt;
        a.zdt = zet[s] * dt;
        a.dtp = dtp;
        a.gam = gam[s];
        a.zet = zet[s];
        a.substage = s;
        if (ctx->c.lrem) {
            // horizontal means of the substage's input T (3dmhdsub.h:297-313), in FP64
            const int e = lrem_profiles32(ctx->g, ctx->c, a.U.p[S_TT], a.bgT, ctx->d_lrem, ctx->stream);
            if (e) return cuda_fail(ctx, (cudaError_t)e, "lRem profiles launch");
        }
        cudaEvent_t* ev = nullptr;
        if (ctx->profiling) {
            if (ctx->prof_used + 2 > ctx->prof_events.size()) {
                for (int j = 0; j < 64; j++) {
                    cudaEvent_t e0;
                    CK(cudaEventCreate(&e0));
                    ctx->prof_events.push_back(e0);
                }
            }
            ev = &ctx->prof_events[ctx->prof_used];
            ctx->prof_used += 2;
            CK(cudaEventRecord(ev[0], ctx->stream));
        }
        int e = fused32_substage(ctx->sw, a, ctx->stream);
        if (e) return cuda_fail(ctx, (cudaError_t)e, "FP32 substage launch");
        if (ev) CK(cudaEventRecord(ev[1], ctx->stream));
        e = fused32_bcon_ghost(ctx->sw, ctx->g, ctx->c, a.Uo, a.Z, a.bgR, a.bgT, ctx->timt, ctx->stream);
        if (e) return cuda_fail(ctx, (cudaError_t)e, "FP32 BCON launch");
        ctx->cur = 1 - ctx->cur;
    }
    return MHD_OK;
}

}  // namespace

int mhd_set_plume(mhd_ctx* ctx, const mhd_plume* pl) {
    if (!ctx || !pl || !pl->EXX || !pl->WYY || !pl->ZEE) return MHD_ERR_INVALID;
    if (!(pl->HH != 0.0)) return fail(ctx, MHD_ERR_INVALID, "HH must be non-zero");
    const int nx = ctx->g.nx, ny = ctx->g.ny, nz = ctx->g.nz;
    if (!ctx->d_plume) {
        if (cudaMalloc(&ctx->d_plume, sizeof(double) * (size_t)(nx + ny + nz)) != cudaSuccess) {
            cudaGetLastError();
            return fail(ctx, MHD_ERR_NOMEM, "plume factor allocation failed");
        }
        ctx->bytes += sizeof(double) * (size_t)(nx + ny + nz);
    }
    // The reference's expressions (3dmhdsub.h:444-458,759-774): CLN uses the
    // float overload of log (its C++ sees <math.h>'s std overloads), the top
    // spot exp(CLN (x - XP)^2), the heat sink exp(CLN (x - XP)^2 / HH).
    const double HH = pl->HH;
    const double CLN = (double)(-4.0f * std::log(2.0f)) / HH / HH;
    const bool sink = ctx->c.pl_mode == 3;
    std::vector<double> h((size_t)(nx + ny + nz), 0.0);
    auto sq = [](double v) { return v * v; };
    for (int x = 0; x < nx; x++) h[x] = sink ? std::exp(CLN * sq(pl->EXX[x] - pl->XP) / HH) : std::exp(CLN * sq(pl->EXX[x] - pl->XP));
    for (int y = 0; y < ny; y++) h[nx + y] = sink ? std::exp(CLN * sq(pl->WYY[y] - pl->YP) / HH) : std::exp(CLN * sq(pl->WYY[y] - pl->YP));
    for (int z = 0; z < nz; z++) h[nx + ny + z] = std::exp(CLN * sq(pl->ZEE[z] - pl->ZP) / HH);
    CK(cudaMemcpyAsync(ctx->d_plume, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->c.plx = ctx->d_plume;
    ctx->c.ply = ctx->d_plume + nx;
    ctx->c.plz = ctx->d_plume + nx + ny;
    ctx->c.pl_hh = HH;
    ctx->pl_TP = ctx->prm.TP;
    ctx->pl_TC = pl->TC;
    ctx->pl_QFH = pl->QFH;
    ctx->pl_OCV = ctx->k.OCV;
    ctx->plume_set = true;
    return ctxops::plume_update(ctx, ctx->timt);
}

namespace mhd::ctxops {
bool plume_time_dependent(const mhd_ctx* c) { return c->c.pl_mode != 0 && c->pl_TC != 0.0; }
int plume_update(mhd_ctx* ctx, double timt) {
    if (ctx->c.pl_mode == 0) return MHD_OK;
    if (!ctx->plume_set)
        return fail(ctx, MHD_ERR_INVALID, "iTCon 2, or TP != 0 with iTCon 0/1, needs mhd_set_plume first");
    const double TP = ctx->pl_TP, TC = ctx->pl_TC;
    if (ctx->c.pl_mode == 3) {
        // 3dmhdsub.h:446-458: TP * OCV [* 0.5 (1 + tanh(log 2 / QFH (TIMT - TC)))]
        ctx->c.pl_s = (TC != 0.0) ? TP * ctx->pl_OCV * 0.5f * (1.0f + std::tanh(std::log(2.0f) / ctx->pl_QFH * (timt - TC)))
                                  : TP * ctx->pl_OCV;
    } else {
        // 3dmhdsub.h:752-757
        ctx->c.pl_tpr = (TC != 0.0) ? TP + (1.0f - TP) * std::exp(-timt / TC) : TP;
    }
    return MHD_OK;
}
FusedArgs fused_args(const mhd_ctx* ctx, int s, double dt, int in) {
    const double gam[3] = {ctx->k.GAM1, ctx->k.GAM2, ctx->k.GAM3};
    const double zet[3] = {ctx->k.ZETA1, ctx->k.ZETA2, 0.0};
    FusedArgs a{};
    a.g = ctx->g;
    a.c = ctx->c;
    a.k = ctx->coef;
    a.U = ::fields_of(ctx, ctx->U[in]);
    a.Uo = ::fields_of(ctx, ctx->U[1 - in]);
    a.Z = ::fields_of(ctx, ctx->Zb);
    a.FT = ctx->Fb ? ctx->Fb + (size_t)F_FT * ctx->ncell : nullptr;
    a.gdt = gam[s] * dt;
    a.zdt = zet[s] * dt;
    a.gam = gam[s];
    a.zet = zet[s];
    a.substage = s;
    return a;
}
void advance_time(mhd_ctx* c, double dt) {
    c->nit += 1;
    c->timc += dt;
    c->timt = c->timi + c->timc;
    c->last_dt = dt;
}
int ensure_u32_1(mhd_ctx* ctx) {
    int rc = ::alloc_f32(ctx, &ctx->U32[1]);
    if (!rc && (ctx->sw & kSwShr) && !ctx->FT64) rc = ::alloc_block(ctx, &ctx->FT64, 1);
    return rc;
}
int sync_zghosts32(mhd_ctx* ctx) { return ::sync_zghosts32(ctx); }
Fields8f fields32_of(const mhd_ctx* c, float* base) { return ::fields32_of(c, base); }
int ensure_u1(mhd_ctx* ctx) { return ::ensure_u1(ctx); }
int sync_zghosts(mhd_ctx* ctx) { return ::sync_zghosts(ctx); }
int alloc_block(mhd_ctx* ctx, double** p, int nfields) { return ::alloc_block(ctx, p, nfields); }
Fields8 fields_of(const mhd_ctx* c, double* base) { return ::fields_of(c, base); }
int fail(mhd_ctx* c, int code, const std::string& msg) { return ::fail(c, code, msg); }
}  // namespace mhd::ctxops

extern "C" {

const char* mhd_status_string(int s) {
    switch (s) {
        case MHD_OK: return "ok";
        case MHD_ERR_INVALID: return "invalid argument";
        case MHD_ERR_UNSUPPORTED: return "unsupported configuration";
        case MHD_ERR_CUDA: return "CUDA error";
        case MHD_ERR_NUMERIC: return "non-finite or non-positive state";
        case MHD_ERR_DT_TOO_SMALL: return "DT too small";
        case MHD_ERR_NOMEM: return "out of device memory";
        case MHD_ERR_TIMEOUT: return "device wait timed out";
        default: return "unknown status";
    }
}

const char* mhd_last_error(const mhd_ctx* ctx) { return ctx ? ctx->err.c_str() : "no context"; }

int mhd_create(const mhd_params* params, void* stream, mhd_ctx** out) {
    if (!out) return MHD_ERR_INVALID;
    *out = nullptr;
    std::string why;
    int rc = validate(params, why);
    if (rc) {
        fprintf(stderr, "mhd_create: %s\n", why.c_str());
        return rc;
    }
    mhd_ctx* ctx = new mhd_ctx();
    ctx->prm = *params;
    const mhd_params& p = ctx->prm;
    compute_constants(p, ctx->k);
    ctx->sw = p.switches & (MHD_SW_LROT | MHD_SW_LMAG | MHD_SW_LSHR);
    ctx->nf = (ctx->sw & MHD_SW_LMAG) ? 8 : 5;
    ctx->g.nx = p.nPx + 2;
    ctx->g.ny = p.nPy + 2;
    ctx->g.nz = p.nPz + 2;
    ctx->g.nPz = p.nPz;
    ctx->g.sy = ctx->g.nx;
    ctx->g.sz = (long long)ctx->g.nx * ctx->g.ny;
    ctx->ncell = (size_t)ctx->g.sz * ctx->g.nz;
    if (stream) {
        ctx->stream = (cudaStream_t)stream;
    } else {
        cudaError_t e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) {
            fprintf(stderr, "mhd_create: %s\n", cudaGetErrorString(e));
            delete ctx;
            return MHD_ERR_CUDA;
        }
        ctx->own_stream = true;
    }
    // metric arrays and the premultiplied coefficients of the fused path
    const int nx = ctx->g.nx, ny = ctx->g.ny, nz = ctx->g.nz;
    std::vector<double> h;
    auto put = [&](const double* a, int n) { h.insert(h.end(), a, a + n); };
    put(p.dxxdx, nx); put(p.d2xxdx2, nx); put(p.DDX, nx);
    put(p.dyydy, ny); put(p.d2yydy2, ny); put(p.DDY, ny);
    put(p.dzzdz, nz); put(p.d2zzdz2, nz); put(p.DDZ, nz);
    put(p.RKAPA, nz); put(p.DKAPA, nz);
    const double hs[3] = {ctx->k.hx, ctx->k.hy, ctx->k.hz};
    const double h2s[3] = {ctx->k.h2x, ctx->k.h2y, ctx->k.h2z};
    const double* d1s[3] = {p.dxxdx, p.dyydy, p.dzzdz};
    const double* d2s[3] = {p.d2xxdx2, p.d2yydy2, p.d2zzdz2};
    const int ns[3] = {nx, ny, nz};
    size_t base_off[3], scaled_off[3];
    for (int ax = 0; ax < 3; ax++) {
        base_off[ax] = h.size();
        for (int i = 0; i < ns[ax]; i++) h.push_back(d1s[ax][i] * hs[ax]);
        for (int i = 0; i < ns[ax]; i++) h.push_back(d2s[ax][i] * hs[ax]);
        for (int i = 0; i < ns[ax]; i++) h.push_back(d1s[ax][i] * d1s[ax][i] * h2s[ax]);
    }
    const double scales[3] = {ctx->k.ORE, ctx->k.ORE * ctx->k.C43, ctx->k.ORM};
    for (int ax = 0; ax < 3; ax++) {
        scaled_off[ax] = h.size();
        for (int sc = 0; sc < 3; sc++) {
            for (int i = 0; i < ns[ax]; i++) h.push_back(d2s[ax][i] * hs[ax] * scales[sc]);
            for (int i = 0; i < ns[ax]; i++) h.push_back(d1s[ax][i] * d1s[ax][i] * h2s[ax] * scales[sc]);
        }
    }
    const size_t kap_off = h.size();
    const double tmpc = ctx->k.OCV / ctx->k.REPR;
    for (int i = 0; i < nz; i++) h.push_back(tmpc * p.RKAPA[i]);
    for (int i = 0; i < nz; i++) h.push_back(tmpc * p.DKAPA[i]);
    for (int i = 0; i < nz; i++) h.push_back(tmpc * p.DKAPA[i] * h[base_off[2] + i]);
    bool uxy = true;
    for (int i = 0; i < nx; i++) uxy = uxy && p.d2xxdx2[i] == 0.0;
    for (int i = 0; i < ny; i++) uxy = uxy && p.d2yydy2[i] == 0.0;
    // ... and the same first-derivative and 'b' coefficients in every interior column
    auto same = [&](size_t off, int n) {
        bool eq = true;
        for (int i = 2; i <= n - 2; i++) eq = eq && h[off + i] == h[off + 1];
        return eq;
    };
    for (int ax = 0; ax < 2 && uxy; ax++) {
        uxy = same(base_off[ax], ns[ax]) && same(base_off[ax] + 2 * (size_t)ns[ax], ns[ax]);
        for (int k = 1; k < 6 && uxy; k += 2) uxy = same(scaled_off[ax] + (size_t)k * ns[ax], ns[ax]);
    }
    // Per-z tables of the fused substage on uniform x / y grids (the x / y
    // coefficients are then the interior column 1's); each records its offset.
    auto push_z = [&](auto value_at) {
        const size_t off = h.size();
        for (int z = 0; z < nz; z++) h.push_back(value_at(z));
        return off;
    };
    auto c1 = [&](int ax, int i) { return h[base_off[ax] + i]; };
    auto c2a = [&](int ax, int i) { return h[base_off[ax] + (size_t)ns[ax] + i]; };
    auto c2b = [&](int ax, int i) { return h[base_off[ax] + 2 * (size_t)ns[ax] + i]; };
    auto s2a = [&](int ax, int k, int i) { return h[scaled_off[ax] + (size_t)(2 * k) * ns[ax] + i]; };
    auto s2b = [&](int ax, int k, int i) { return h[scaled_off[ax] + (size_t)(2 * k + 1) * ns[ax] + i]; };
    size_t lapS_off[6], condT_off[5], lapZ_off[8];
    // S = 2 (sx + sy + sz) of the Laplacians of u, v, w (viscous scales, C43 on the x, y, z
    // axis), T (unscaled), B (resistive), and 2 (sx + sy) of B on the wall planes
    {
        const int kx[6] = {1, 0, 0, -1, 2, 2}, ky[6] = {0, 1, 0, -1, 2, 2}, kz[6] = {0, 0, 1, -1, 2, -2};
        for (int set = 0; set < 6; set++)
            lapS_off[set] = push_z([&](int z) {
                const double sx = kx[set] < 0 ? c2b(0, 1) : s2b(0, kx[set], 1);
                const double sy = ky[set] < 0 ? c2b(1, 1) : s2b(1, ky[set], 1);
                const double sz = kz[set] == -2 ? 0.0 : kz[set] < 0 ? c2b(2, z) : s2b(2, kz[set], z);
                return 2.0 * (sx + sy + sz);
            });
    }
    // the viscous cross-term factors C13*ORE*cx1*cz1, C13*ORE*cy1*cz1 (the kernel's order)
    const double c13ore = ctx->k.C13 * ctx->k.ORE;
    const double kx13 = c13ore * c1(0, 1), ky13 = c13ore * c1(1, 1);
    const size_t kxz_off = push_z([&](int z) { return kx13 * c1(2, z); });
    const size_t kyz_off = push_z([&](int z) { return ky13 * c1(2, z); });
    const size_t ocz1_off = push_z([&](int z) { return ctx->k.OBETA * c1(2, z); });
    // conduction with kapz folded in: kapz cx2b, kapz cy2b, the factors of T(z+1) and
    // T(z-1) kapz (cz2b +- cz2a) +- dkapz cz1, and kapz S_T
    {
        auto kz = [&](int z) { return h[kap_off + z]; };
        auto dkz = [&](int z) { return h[kap_off + nz + z]; };
        condT_off[0] = push_z([&](int z) { return kz(z) * c2b(0, 1); });
        condT_off[1] = push_z([&](int z) { return kz(z) * c2b(1, 1); });
        condT_off[2] = push_z([&](int z) { return kz(z) * (c2b(2, z) + c2a(2, z)) + dkz(z) * c1(2, z); });
        condT_off[3] = push_z([&](int z) { return kz(z) * (c2b(2, z) - c2a(2, z)) - dkz(z) * c1(2, z); });
        condT_off[4] = push_z([&](int z) { return kz(z) * (2.0 * (c2b(0, 1) + c2b(1, 1) + c2b(2, z))); });
    }
    // z second-derivative factors b + a and b - a of the planes above and below, for the
    // scale pairs k = 0, 1, 2 (ORE, ORE*C43, ORM) and unscaled (k = 3)
    for (int k = 0; k < 4; k++) {
        auto za = [&](int z) { return k < 3 ? s2a(2, k, z) : c2a(2, z); };
        auto zb = [&](int z) { return k < 3 ? s2b(2, k, z) : c2b(2, z); };
        lapZ_off[2 * k] = push_z([&](int z) { return zb(z) + za(z); });
        lapZ_off[2 * k + 1] = push_z([&](int z) { return zb(z) - za(z); });
    }
    if (cudaMalloc(&ctx->d_metric, h.size() * sizeof(double)) != cudaSuccess ||
        cudaMemcpyAsync(ctx->d_metric, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, ctx->stream) !=
            cudaSuccess) {
        cudaGetLastError();
        mhd_destroy(ctx);
        return MHD_ERR_NOMEM;
    }
    ctx->bytes += h.size() * sizeof(double);
    const double* m = ctx->d_metric;
    Consts& c = ctx->c;
    c.dxxdx = m; c.d2xxdx2 = m + nx; c.DDX = m + 2 * nx; m += 3 * nx;
    c.dyydy = m; c.d2yydy2 = m + ny; c.DDY = m + 2 * ny; m += 3 * ny;
    c.dzzdz = m; c.d2zzdz2 = m + nz; c.DDZ = m + 2 * nz; c.RKAPA = m + 3 * nz; c.DKAPA = m + 4 * nz; m += 5 * nz;
    {
        const double* b0 = ctx->d_metric;
        const double** c1s[3] = {&ctx->coef.cx1, &ctx->coef.cy1, &ctx->coef.cz1};
        const double** c2as[3] = {&ctx->coef.cx2a, &ctx->coef.cy2a, &ctx->coef.cz2a};
        const double** c2bs[3] = {&ctx->coef.cx2b, &ctx->coef.cy2b, &ctx->coef.cz2b};
        for (int ax = 0; ax < 3; ax++) {
            *c1s[ax] = b0 + base_off[ax];
            *c2as[ax] = b0 + base_off[ax] + ns[ax];
            *c2bs[ax] = b0 + base_off[ax] + 2 * ns[ax];
            for (int k = 0; k < 6; k++) ctx->coef.s2[ax][k] = b0 + scaled_off[ax] + (size_t)k * ns[ax];
        }
        ctx->coef.kapz = b0 + kap_off;
        ctx->coef.dkapz = b0 + kap_off + nz;
        ctx->coef.dkz = b0 + kap_off + 2 * (size_t)nz;
        ctx->coef.uniform_xy = uxy ? 1 : 0;
        ctx->coef.isotropic_xy = (uxy && c1(0, 1) == c1(1, 1)) ? 1 : 0;
        for (int set = 0; set < 6; set++) ctx->coef.lapS[set] = b0 + lapS_off[set];
        ctx->coef.kxz = b0 + kxz_off;
        ctx->coef.kyz = b0 + kyz_off;
        ctx->coef.ocz1 = b0 + ocz1_off;
        for (int t = 0; t < 5; t++) ctx->coef.condT[t] = b0 + condT_off[t];
        for (int t = 0; t < 8; t++) ctx->coef.lapZ[t] = b0 + lapZ_off[t];
    }
    c.C13 = ctx->k.C13; c.C23 = ctx->k.C23; c.C43 = ctx->k.C43;
    c.hx = ctx->k.hx; c.h2x = ctx->k.h2x; c.hy = ctx->k.hy; c.h2y = ctx->k.h2y; c.hz = ctx->k.hz; c.h2z = ctx->k.h2z;
    c.GRAV = p.GRAV; c.THETA = p.THETA; c.RE = p.RE; c.REPR = ctx->k.REPR; c.ORE = ctx->k.ORE;
    c.OCV = ctx->k.OCV; c.CV = ctx->k.CV; c.GAMMA = p.GAMMA; c.OMX = ctx->k.OMX; c.OMZ = ctx->k.OMZ;
    c.RM = p.RM; c.ORM = ctx->k.ORM; c.OBETA = ctx->k.OBETA; c.TB = p.TB; c.TP = p.TP; c.SFF = p.SFF;
    c.DDXmin = HUGE_VAL;
    for (int x = 1; x <= nx - 2; x++) c.DDXmin = (p.DDX[x] < c.DDXmin) ? p.DDX[x] : c.DDXmin;
    c.izCon = p.izCon; c.iTCon = p.iTCon; c.iBCon = p.iBCon;
    c.lrem = (p.switches & MHD_SW_LREM) ? 1 : 0;
    c.TU = p.TU; c.DZTU = p.DZTU; c.DZTB = p.DZTB;
    // plume terms (their parameters come with mhd_set_plume)
    c.pl_mode = (p.iTCon == 2) ? 3 : (p.TP != 0.0 && p.iTCon == 0) ? 1 : (p.TP != 0.0 && p.iTCon == 1) ? 2 : 0;

    ctx->red_blocks = 152 * 8;
    ctx->fp32 = p.precision == MHD_PREC_FP32;
    ctx->h_cz.assign(h.begin() + base_off[2], h.begin() + base_off[2] + 3 * nz);
    ctx->h_bg.assign(4 * (size_t)nz, 0.0);
    int arc = MHD_OK;
    if (ctx->fp32) {
        arc = alloc_f32(ctx, &ctx->U32[0]);
        // 4 x nz double profiles, then the [kZfRows][nz] float coefficient table
        const size_t bg_bytes = sizeof(double) * 4 * nz + sizeof(float) * kZfRows * nz;
        if (!arc && cudaMalloc(&ctx->d_bg, bg_bytes) != cudaSuccess) arc = MHD_ERR_NOMEM;
        if (!arc && cudaMemsetAsync(ctx->d_bg, 0, bg_bytes, ctx->stream) != cudaSuccess) arc = MHD_ERR_CUDA;
        ctx->h_zf.assign(kZfRows * (size_t)nz, 0.0f);
        for (int z = 0; z < nz; z++) {
            for (int r = 0; r < 3; r++) ctx->h_zf[(size_t)r * nz + z] = (float)ctx->h_cz[(size_t)r * nz + z];
            ctx->h_zf[5 * (size_t)nz + z] = (float)p.RKAPA[z];
            ctx->h_zf[6 * (size_t)nz + z] = (float)p.DKAPA[z];
        }
        if (!arc && cudaMemcpyAsync(ctx->d_bg + 4 * nz, ctx->h_zf.data(), sizeof(float) * kZfRows * nz,
                                    cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess) arc = MHD_ERR_CUDA;
    } else {
        arc = alloc_block(ctx, &ctx->U[0], 8);
    }
    if (!arc) arc = alloc_block(ctx, &ctx->Zb, 8);
    if (!arc && ctx->fp32 && (ctx->sw & kSwShr)) arc = alloc_block(ctx, &ctx->FT64, 1);
    if (!arc && cudaMalloc(&ctx->red, sizeof(double) * 8 * (size_t)ctx->red_blocks) != cudaSuccess) arc = MHD_ERR_NOMEM;
    if (!arc && c.lrem) {
        if (cudaMalloc(&ctx->d_lrem, sizeof(double) * 3 * nz) != cudaSuccess) arc = MHD_ERR_NOMEM;
        else {
            ctx->bytes += sizeof(double) * 3 * nz;
            c.lrem_ttm = ctx->d_lrem;
            c.lrem_hrad = ctx->d_lrem + nz;
            c.lrem_g = ctx->d_lrem + 2 * nz;
        }
    }
    // d_out: 8 doubles of reduction results, then the kDtRecord-double time-step record
    if (!arc && cudaMalloc(&ctx->d_out, sizeof(double) * (8 + kDtRecord)) != cudaSuccess) arc = MHD_ERR_NOMEM;
    if (!arc && cudaMallocHost(&ctx->h_out, sizeof(double) * (8 + kDtRecord)) != cudaSuccess) arc = MHD_ERR_NOMEM;
    if (arc) {
        cudaGetLastError();
        fprintf(stderr, "mhd_create: %s\n", ctx->err.empty() ? "allocation failed" : ctx->err.c_str());
        mhd_destroy(ctx);
        return MHD_ERR_NOMEM;
    }
    ctx->bytes += sizeof(double) * (8 * (size_t)ctx->red_blocks + 8 + kDtRecord);
    ctx->timt = ctx->timi = ctx->timc = 0.0;
    ctx->nit = 0;
    // the uploads and clears above are ordered on the context's stream; finish
    // them before the host tables go away and before other streams read them
    if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
        cudaGetLastError();
        fprintf(stderr, "mhd_create: the set-up copies failed\n");
        mhd_destroy(ctx);
        return MHD_ERR_CUDA;
    }
    *out = ctx;
    return MHD_OK;
}

int mhd_destroy(mhd_ctx* ctx) {
    if (!ctx) return MHD_ERR_INVALID;
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    cudaFree(ctx->d_metric);
    cudaFree(ctx->U[0]);
    cudaFree(ctx->U[1]);
    cudaFree(ctx->Zb);
    cudaFree(ctx->Fb);
    cudaFree(ctx->Sb);
    cudaFree(ctx->red);
    cudaFree(ctx->d_out);
    cudaFree(ctx->U32[0]);
    cudaFree(ctx->U32[1]);
    cudaFree(ctx->FT64);
    cudaFree(ctx->d_bg);
    cudaFree(ctx->d_plume);
    cudaFree(ctx->d_lrem);
    if (ctx->h_out) cudaFreeHost(ctx->h_out);
    if (ctx->t0) cudaEventDestroy(ctx->t0);
    if (ctx->t1) cudaEventDestroy(ctx->t1);
    for (cudaEvent_t e : ctx->prof_events) cudaEventDestroy(e);
    for (cudaEvent_t e : ctx->slab_events) cudaEventDestroy(e);
    if (ctx->s_up) cudaStreamDestroy(ctx->s_up);
    if (ctx->s_down) cudaStreamDestroy(ctx->s_down);
    for (cudaStream_t st : ctx->s_sub)
        if (st) cudaStreamDestroy(st);
    if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return MHD_OK;
}

int mhd_get_constants(const mhd_ctx* ctx, mhd_constants* out) {
    if (!ctx || !out) return MHD_ERR_INVALID;
    *out = ctx->k;
    return MHD_OK;
}

int mhd_compute_constants(const mhd_params* params, mhd_constants* out) {
    if (!params || !out) return MHD_ERR_INVALID;
    compute_constants(*params, *out);
    return MHD_OK;
}

int mhd_device_bytes(const mhd_ctx* ctx, size_t* out) {
    if (!ctx || !out) return MHD_ERR_INVALID;
    *out = ctx->bytes;
    return MHD_OK;
}

static double* field_ptr(mhd_ctx* ctx, int field, bool for_write, int* rc) {
    *rc = MHD_OK;
    if (field < 0 || field >= MHD_NFIELDS) {
        *rc = fail(ctx, MHD_ERR_INVALID, "field id out of range");
        return nullptr;
    }
    if (field < 8) {
        if (for_write) ctx->ghosts_synced = false;
        return ctx->U[ctx->cur] + (size_t)field * ctx->ncell;
    }
    if (ctx->fp32 && field < 16) {
        if (field != MHD_FT || !ctx->FT64) {
            *rc = fail(ctx, MHD_ERR_UNSUPPORTED, "an FP32-storage context keeps only FT (with lShr) of the right-hand sides");
            return nullptr;
        }
        return ctx->FT64;
    }
    if (field < 16) {
        *rc = alloc_block(ctx, &ctx->Fb, 8);
        return *rc ? nullptr : ctx->Fb + (size_t)(field - 8) * ctx->ncell;
    }
    return ctx->Zb + (size_t)(field - 16) * ctx->ncell;
}

int mhd_upload(mhd_ctx* ctx, int field, const double* host) {
    if (!ctx || !host) return MHD_ERR_INVALID;
    if (ctx->fp32 && field >= 0 && field < 8) return upload32(ctx, field, host);
    int rc;
    double* d = field_ptr(ctx, field, true, &rc);
    if (!d) return rc;
    CK(cudaMemcpyAsync(d, host, field_bytes(ctx), cudaMemcpyHostToDevice, ctx->stream));
    return MHD_OK;
}

int mhd_download(mhd_ctx* ctx, int field, double* host) {
    if (!ctx || !host) return MHD_ERR_INVALID;
    if (ctx->fp32 && field >= 0 && field < 8) return download32(ctx, field, host);
    int rc;
    double* d = field_ptr(ctx, field, false, &rc);
    if (!d) return rc;
    CK(cudaMemcpyAsync(host, d, field_bytes(ctx), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return MHD_OK;
}

int mhd_upload_state(mhd_ctx* ctx, const double* host) {
    if (!ctx || !host) return MHD_ERR_INVALID;
    if (ctx->fp32) {
        for (int f = 0; f < ctx->nf; f++) {
            int rc = upload32(ctx, f, host + (size_t)f * ctx->ncell);
            if (rc) return rc;
        }
        return MHD_OK;
    }
    ctx->ghosts_synced = false;
    CK(cudaMemcpyAsync(ctx->U[ctx->cur], host, field_bytes(ctx) * ctx->nf, cudaMemcpyHostToDevice, ctx->stream));
    return MHD_OK;
}

int mhd_download_state(mhd_ctx* ctx, double* host) {
    if (!ctx || !host) return MHD_ERR_INVALID;
    if (ctx->fp32) {
        for (int f = 0; f < ctx->nf; f++) {
            int rc = download32(ctx, f, host + (size_t)f * ctx->ncell);
            if (rc) return rc;
        }
        return MHD_OK;
    }
    CK(cudaMemcpyAsync(host, ctx->U[ctx->cur], field_bytes(ctx) * ctx->nf, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return MHD_OK;
}

int mhd_set_time(mhd_ctx* ctx, double timt, long long nit) {
    if (!ctx) return MHD_ERR_INVALID;
    // a restart: TIMI = the restored time, TIMC counts from 0 (3dmhd.cpp:114,460)
    ctx->timt = timt;
    ctx->timi = timt;
    ctx->timc = 0.0;
    ctx->nit = nit;
    return MHD_OK;
}

int mhd_fluxes(mhd_ctx* ctx) {
    if (!ctx) return MHD_ERR_INVALID;
    if (ctx->fp32) return fail(ctx, MHD_ERR_UNSUPPORTED, "the unfused calls work on FP64 state only");
    int rc = ensure_parity_buffers(ctx);
    if (!rc) rc = ctxops::plume_update(ctx, ctx->timt);
    if (rc) return rc;
    if (ctx->c.lrem) {
        // lRem: the wall ghost planes of RO take the second interior plane
        // (3dmhdsub.h:229-238), and the horizontal means of T in the
        // reference's summation order (3dmhdsub.h:297-301,698-718)
        double* RO = ctx->U[ctx->cur] + (size_t)S_RO * ctx->ncell;
        const size_t plane = (size_t)ctx->g.sz;
        CK(cudaMemcpyAsync(RO, RO + 2 * plane, plane * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
        CK(cudaMemcpyAsync(RO + (size_t)(ctx->g.nz - 1) * plane, RO + (size_t)(ctx->g.nz - 3) * plane,
                           plane * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
        const int e = lrem_profiles(ctx->g, ctx->c, ctx->U[ctx->cur] + (size_t)S_TT * ctx->ncell, ctx->d_lrem, true,
                                    ctx->stream);
        if (e) return cuda_fail(ctx, (cudaError_t)e, "lRem profiles launch");
    }
    double* S = ctx->Sb;
    ctx->ghosts_synced = false;  // 1/rho is written into RO over every cell, wall ghost planes included
    const int e = parity_fluxes(ctx->sw, ctx->g, ctx->c, fields_of(ctx, ctx->U[ctx->cur]), fields_of(ctx, ctx->Fb), S,
                                S + ctx->ncell, S + 2 * ctx->ncell, S + 3 * ctx->ncell, ctx->stream);
    if (e) return cuda_fail(ctx, (cudaError_t)e, "fluxes launch");
    return MHD_OK;
}

static int rk(mhd_ctx* ctx, int kind, double coef) {
    if (!ctx) return MHD_ERR_INVALID;
    if (ctx->fp32) return fail(ctx, MHD_ERR_UNSUPPORTED, "the unfused calls work on FP64 state only");
    int rc = alloc_block(ctx, &ctx->Fb, 8);
    if (rc) return rc;
    if (kind == 2) ctx->ghosts_synced = false;
    const int e = parity_rk(kind, ctx->nf, ctx->g, fields_of(ctx, ctx->U[ctx->cur]), fields_of(ctx, ctx->Zb),
                            fields_of(ctx, ctx->Fb), coef, ctx->stream);
    if (e) return cuda_fail(ctx, (cudaError_t)e, "RK launch");
    return MHD_OK;
}

int mhd_rk_zeta0(mhd_ctx* ctx) { return rk(ctx, 0, 0.0); }
int mhd_rk_zeta(mhd_ctx* ctx, double coef) { return rk(ctx, 1, coef); }
int mhd_rk_gam(mhd_ctx* ctx, double coef) { return rk(ctx, 2, coef); }

int mhd_bcon(mhd_ctx* ctx, double timt) {
    if (!ctx) return MHD_ERR_INVALID;
    if (ctx->fp32) return fail(ctx, MHD_ERR_UNSUPPORTED, "the unfused calls work on FP64 state only");
    const int rc = ctxops::plume_update(ctx, timt);
    if (rc) return rc;
    const int e = parity_bcon(ctx->sw, ctx->g, ctx->c, fields_of(ctx, ctx->U[ctx->cur]), timt, ctx->stream);
    if (e) return cuda_fail(ctx, (cudaError_t)e, "BCON launch");
    return MHD_OK;
}

int mhd_communicate(mhd_ctx* ctx) {
    if (!ctx) return MHD_ERR_INVALID;
    ctx->ghosts_synced = false;
    if (ctx->fp32) {
        const int e = communicate32(ctx->nf, ctx->g, fields32_of(ctx, ctx->U32[ctx->cur]), ctx->stream);
        if (e) return cuda_fail(ctx, (cudaError_t)e, "communicate launch");
        return MHD_OK;
    }
    const int e = parity_communicate(ctx->nf, ctx->g, fields_of(ctx, ctx->U[ctx->cur]), ctx->stream);
    if (e) return cuda_fail(ctx, (cudaError_t)e, "communicate launch");
    return MHD_OK;
}

int mhd_cfl_dt(mhd_ctx* ctx, double* dt, double* umach) {
    if (!ctx) return MHD_ERR_INVALID;
    const bool mag = (ctx->sw & kSwMag) != 0;
    const int nz = ctx->g.nz;
    int e = ctx->fp32 ? cfl32_rows(mag, ctx->g, ctx->c, fields32_of(ctx, ctx->U32[ctx->cur]), ctx->d_bg,
                                   ctx->d_bg + nz, ctx->red, ctx->red_blocks, ctx->d_out, ctx->stream)
                      : parity_cfl(mag, ctx->g, ctx->c, fields_of(ctx, ctx->U[ctx->cur]), ctx->red, ctx->red_blocks,
                                   ctx->d_out, ctx->stream);
    if (e) return cuda_fail(ctx, (cudaError_t)e, "CFL launch");
    CK(cudaMemcpyAsync(ctx->h_out, ctx->d_out, sizeof(double) * 5, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    const double* o = ctx->h_out;
    auto mn = [](double a, double b) { return (b < a) ? b : a; };
    // 3dmhdsub.h:44,102-104
    const double d = mag ? ctx->prm.SFF * mn(mn(o[1], o[2]), mn(o[3], o[4])) : ctx->prm.SFF * mn(mn(o[1], o[2]), o[3]);
    ctx->last_umach = std::sqrt(o[0]);
    if (umach) *umach = ctx->last_umach;
    if (dt) *dt = d;
    if (!(d == d) || !(o[0] == o[0])) return fail(ctx, MHD_ERR_NUMERIC, "non-finite CFL estimate");
    return MHD_OK;
}

static int parity_step(mhd_ctx* ctx, double dt) {
    const double g[3] = {ctx->k.GAM1, ctx->k.GAM2, ctx->k.GAM3};
    const double zt[2] = {ctx->k.ZETA1, ctx->k.ZETA2};
    int rc;
    for (int s = 0; s < 3; s++) {
        rc = s == 0 ? mhd_rk_zeta0(ctx) : mhd_rk_zeta(ctx, zt[s - 1] * dt);
        if (rc) return rc;
        if ((rc = mhd_fluxes(ctx))) return rc;
        if ((rc = mhd_rk_gam(ctx, g[s] * dt))) return rc;
        if ((rc = mhd_bcon(ctx, ctx->timt))) return rc;
        if ((rc = mhd_communicate(ctx))) return rc;
    }
    return MHD_OK;
}

int mhd_step(mhd_ctx* ctx, double dt, mhd_diag* out) {
    if (!ctx) return MHD_ERR_INVALID;
    int rc;
    if (!(dt > 0.0)) {
        rc = mhd_cfl_dt(ctx, &dt, nullptr);
        if (rc) return rc;
        if (dt < 1.0e-8f) return fail(ctx, MHD_ERR_DT_TOO_SMALL, "DT too small, halt (3dmhd.cpp:292-331)");
    }
    rc = ctxops::plume_update(ctx, ctx->timt);
    if (rc) return rc;
    rc = ctx->fp32 ? fused32_step(ctx, dt) : ctx->prm.path == MHD_PATH_PARITY ? parity_step(ctx, dt) : fused_step(ctx, dt);
    if (rc) return rc;
    ctxops::advance_time(ctx, dt);
    if (out) {
        memset(out, 0, sizeof(*out));
        out->dt = dt;
        out->umach = ctx->last_umach;
        out->timt = ctx->timt;
        out->nit = ctx->nit;
    }
    return MHD_OK;
}

int mhd_steps(mhd_ctx* ctx, int n, double dt) {
    if (!ctx || n < 0 || !(dt > 0.0)) return MHD_ERR_INVALID;
    for (int s = 0; s < n; s++) {
        int rc = mhd_step(ctx, dt, nullptr);
        if (rc) return rc;
    }
    return MHD_OK;
}

int mhd_steps_cfl(mhd_ctx* ctx, int n, mhd_diag* out) {
    if (!ctx || n < 0) return MHD_ERR_INVALID;
    if (out) memset(out, 0, sizeof(*out));
    if (ctx->prm.path == MHD_PATH_PARITY || ctxops::plume_time_dependent(ctx)) {
        // these read the CFL dt back every step (the unfused sequence takes
        // host scalars; a time-dependent plume needs TIMT on the host)
        mhd_diag d{};
        for (int s = 0; s < n; s++) {
            const int rc = mhd_step(ctx, 0.0, &d);
            if (out) *out = d;
            if (rc) return rc;
        }
        return MHD_OK;
    }
    if (int rp = ctxops::plume_update(ctx, ctx->timt)) return rp;
    double* rec = ctx->d_out + 8;
    double* h = ctx->h_out + 8;
    for (int k = 0; k < kDtRecord; k++) h[k] = 0.0;
    h[1] = ctx->timt;
    h[6] = ctx->timi;
    h[7] = ctx->timc;
    CK(cudaMemcpyAsync(rec, h, sizeof(double) * kDtRecord, cudaMemcpyHostToDevice, ctx->stream));
    const bool mag = (ctx->sw & kSwMag) != 0;
    const int nz = ctx->g.nz;
    for (int s = 0; s < n; s++) {
        int e;
        if (ctx->fp32) {
            e = cfl32_dt_on_device(mag, ctx->g, ctx->c, fields32_of(ctx, ctx->U32[ctx->cur]), ctx->d_bg,
                                   ctx->d_bg + nz, ctx->red, ctx->red_blocks, rec, ctx->stream);
        } else {
            int rc = ensure_u1(ctx);
            if (!rc) rc = sync_zghosts(ctx);
            if (rc) return rc;
            e = cfl_dt_on_device(mag, ctx->g, ctx->c, fields_of(ctx, ctx->U[ctx->cur]), ctx->red, ctx->red_blocks,
                                 rec, ctx->stream);
        }
        if (e) return cuda_fail(ctx, (cudaError_t)e, "CFL launch");
        // BCON reads TIMT only through cos(0 * TIMT) = 1 (3dmhdsub.h:725,732,824), so the
        // host's TIMT at the call stands in for the device's
        const int rc = ctx->fp32 ? fused32_step(ctx, 0.0, rec) : fused_step(ctx, 0.0, rec);
        if (rc) return rc;
    }
    CK(cudaMemcpyAsync(h, rec, sizeof(double) * kDtRecord, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    const long long done = (long long)h[5];
    ctx->timt = h[1];
    ctx->timc = h[7];
    ctx->nit += done;
    ctx->last_umach = h[2];
    if (done > 0 || h[3] != 0.0) ctx->last_dt = h[4];
    if (out) {
        out->dt = ctx->last_dt;
        out->umach = ctx->last_umach;
        out->timt = ctx->timt;
        out->nit = ctx->nit;
    }
    if (h[3] != 0.0) {
        if (!(h[4] == h[4]) || !(h[2] == h[2])) return fail(ctx, MHD_ERR_NUMERIC, "non-finite CFL estimate");
        return fail(ctx, MHD_ERR_DT_TOO_SMALL,
                    "DT too small, halt after step " + std::to_string(ctx->nit) + " (3dmhd.cpp:292-331)");
    }
    return MHD_OK;
}

int mhd_diagnostics(mhd_ctx* ctx, mhd_diag* out) {
    if (!ctx || !out) return MHD_ERR_INVALID;
    const bool mag = (ctx->sw & kSwMag) != 0;
    const int nz = ctx->g.nz;
    int e = ctx->fp32 ? diag32(mag, ctx->g, ctx->c, fields32_of(ctx, ctx->U32[ctx->cur]), ctx->d_bg, ctx->d_bg + nz,
                               ctx->red, ctx->red_blocks, ctx->d_out, ctx->stream)
                      : diag_reduce(mag, ctx->g, ctx->c, fields_of(ctx, ctx->U[ctx->cur]), ctx->red, ctx->red_blocks,
                                    ctx->d_out, ctx->stream);
    if (e) return cuda_fail(ctx, (cudaError_t)e, "diagnostics launch");
    CK(cudaMemcpyAsync(ctx->h_out, ctx->d_out, sizeof(double) * 4, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    memset(out, 0, sizeof(*out));
    out->total_mass = ctx->h_out[0];
    out->total_energy = ctx->h_out[1];
    out->max_divb = ctx->h_out[2];
    out->flags = (int)ctx->h_out[3];
    out->dt = ctx->last_dt;
    out->umach = ctx->last_umach;
    out->timt = ctx->timt;
    out->nit = ctx->nit;
    return out->flags ? fail(ctx, MHD_ERR_NUMERIC, "state has non-finite or non-positive values") : MHD_OK;
}

int mhd_sync(mhd_ctx* ctx) {
    if (!ctx) return MHD_ERR_INVALID;
    CK(cudaStreamSynchronize(ctx->stream));
    return MHD_OK;
}

int mhd_set_device(int device) {
    return cudaSetDevice(device) == cudaSuccess ? MHD_OK : MHD_ERR_CUDA;
}

int mhd_timer_start(mhd_ctx* ctx) {
    if (!ctx) return MHD_ERR_INVALID;
    if (!ctx->t0) CK(cudaEventCreate(&ctx->t0));
    if (!ctx->t1) CK(cudaEventCreate(&ctx->t1));
    CK(cudaEventRecord(ctx->t0, ctx->stream));
    return MHD_OK;
}

int mhd_timer_stop(mhd_ctx* ctx, double* ms) {
    if (!ctx || !ms || !ctx->t0) return MHD_ERR_INVALID;
    CK(cudaEventRecord(ctx->t1, ctx->stream));
    CK(cudaEventSynchronize(ctx->t1));
    float f = 0.f;
    CK(cudaEventElapsedTime(&f, ctx->t0, ctx->t1));
    *ms = (double)f;
    return MHD_OK;
}

int mhd_profile(mhd_ctx* ctx, int enable) {
    if (!ctx) return MHD_ERR_INVALID;
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->profiling = enable != 0;
    ctx->prof_used = 0;
    return MHD_OK;
}

int mhd_profile_read(mhd_ctx* ctx, double* substage_ms, long long* launches) {
    if (!ctx) return MHD_ERR_INVALID;
    CK(cudaStreamSynchronize(ctx->stream));
    double tot = 0.0;
    for (size_t j = 0; j + 1 < ctx->prof_used; j += 2) {
        float f = 0.f;
        CK(cudaEventElapsedTime(&f, ctx->prof_events[j], ctx->prof_events[j + 1]));
        tot += f;
    }
    if (substage_ms) *substage_ms = tot;
    if (launches) *launches = (long long)(ctx->prof_used / 2);
    return MHD_OK;
}

int mhd_fp64_peak(double* tflops) {
    if (!tflops) return MHD_ERR_INVALID;
    return fp64_peak(tflops) == 0 ? MHD_OK : MHD_ERR_CUDA;
}

int mhd_host_alloc(size_t bytes, void** out) {
    if (!out) return MHD_ERR_INVALID;
    return cudaMallocHost(out, bytes) == cudaSuccess ? MHD_OK : MHD_ERR_NOMEM;
}

int mhd_host_free(void* p) { return cudaFreeHost(p) == cudaSuccess ? MHD_OK : MHD_ERR_CUDA; }

}  // extern "C"
