// mhd_context.h -- the context behind mhd_ctx* (private to the library).
#pragma once

#include "../../include/mhd_gb300.h"
#include "mhd_common.cuh"

#include <string>
#include <vector>

using namespace mhd;

struct mhd_ctx {
    mhd_params prm{};
    mhd_constants k{};
    Grid g{};
    Consts c{};
    Coefs coef{};
    unsigned sw = 0;
    int nf = 5;
    size_t ncell = 0;  // nx*ny*nz
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    double* d_metric = nullptr;  // 11 metric arrays + 9 coefficient arrays
    double* U[2] = {nullptr, nullptr};
    int cur = 0;
    double* Zb = nullptr;
    double* Fb = nullptr;
    double* Sb = nullptr;
    double* red = nullptr;   // reduction partials
    double* d_out = nullptr; // 8 doubles of reduction results
    double* h_out = nullptr; // pinned mirror of d_out
    int red_blocks = 0;
    bool ghosts_synced = false;  // z ghost planes of U[1-cur] match U[cur]
    // simulation time as step() keeps it (3dmhdsub.h:150-152): TIMC sums the
    // steps' DT, TIMT = TIMI + TIMC
    double timt = 0.0, timi = 0.0, timc = 0.0;
    long long nit = 0;
    double last_dt = 0.0, last_umach = 0.0;
    size_t bytes = 0;
    std::string err;
    // FP32-storage contexts
    bool fp32 = false;
    float* U32[2] = {nullptr, nullptr};
    double* FT64 = nullptr;     // persistent FT (lShr)
    double* d_bg = nullptr;     // rho0, T0, dzT0, d2zT0 (4 x nz), then the float table
    std::vector<double> h_bg;   // host copy of the four profiles
    std::vector<double> h_cz;   // cz1, cz2a, cz2b (3 x nz)
    // float per-z coefficients of the FP32 kernels, [kZfRows][nz]: cz1, cz2a,
    // cz2b, dzT0, d2zT0, RKAPA, DKAPA, the profiles' hydrostatic residual
    // rho0 GRAV - D_z(rho0 T0), and rho0, T0 as float pairs hi, lo (device
    // copy after d_bg's 4 x nz doubles)
    std::vector<float> h_zf;
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    bool profiling = false;
    std::vector<cudaEvent_t> prof_events;  // pairs around each substage launch
    size_t prof_used = 0;
    // plume terms: parameters from mhd_set_plume, Gaussian factors on the device
    bool plume_set = false;
    double pl_TP = 0.0, pl_TC = 0.0, pl_QFH = 0.0, pl_OCV = 0.0;
    double* d_plume = nullptr;  // plx (nx), ply (ny), plz (nz)
    double* d_lrem = nullptr;   // lRem: TTM, HRAD, G (3 x nz)
    // host-to-host steps: copy streams, one compute stream per RK3 substage and
    // per-slab events (created on first use)
    cudaStream_t s_up = nullptr, s_down = nullptr;
    cudaStream_t s_sub[3] = {nullptr, nullptr, nullptr};
    std::vector<cudaEvent_t> slab_events;
};

namespace mhd::ctxops {
int ensure_u32_1(mhd_ctx* ctx);
int sync_zghosts32(mhd_ctx* ctx);
Fields8f fields32_of(const mhd_ctx* c, float* base);
int ensure_u1(mhd_ctx* ctx);
int sync_zghosts(mhd_ctx* ctx);
int alloc_block(mhd_ctx* ctx, double** p, int nfields);
Fields8 fields_of(const mhd_ctx* c, double* base);
int fail(mhd_ctx* c, int code, const std::string& msg);
// one completed step of length dt: nIt, TIMC and TIMT advance as 3dmhdsub.h:150-152
void advance_time(mhd_ctx* c, double dt);
// refresh the time-dependent plume scalars for simulation time timt; fails
// when the context needs plume parameters that mhd_set_plume has not given
int plume_update(mhd_ctx* c, double timt);
// whether the plume terms depend on the simulation time (TC != 0)
bool plume_time_dependent(const mhd_ctx* c);
// FP32 contexts: with rho0(z), T0(z) in h_bg, derive T0's z derivatives and
// the float coefficient table and upload the profiles
int profiles_from_means(mhd_ctx* c);
// FusedArgs of substage s (0..2) of the fused FP64 step reading state buffer
// U[in] and writing U[1-in]
FusedArgs fused_args(const mhd_ctx* c, int s, double dt, int in);
}  // namespace mhd::ctxops
