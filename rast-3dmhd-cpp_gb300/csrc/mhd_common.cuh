// mhd_common.cuh -- device-side definitions shared by the 3dmhd kernels.
//
// Layout of every field: double (or float) [nz][ny][nx], x fastest, one ghost
// cell per side, exactly the reference's `data` type (3dmhddata.h:8) on one
// global domain.  Strides: sy = nx, sz = nx*ny (elements).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace mhd {

// Compile-time physics switches, the reference's 3dmhdparam.h:8-17 and
// :86-107 macros as template parameters.  Horizontal boundaries are periodic
// only (fluxes() exits otherwise, 3dmhdsub.h:204-209); lPot is never read by
// the reference; lRem is out of scope.
template <bool MAG, bool ROT, bool SHR>
struct Switches {
    static constexpr bool lMag = MAG;
    static constexpr bool lRot = ROT;
    static constexpr bool lShr = SHR;
    static constexpr bool lPot = false;
    static constexpr bool lRem = false;
    static constexpr int ixCon = 0;
    static constexpr int iyCon = 0;
};

// field slots of the state (dump record order, 3dmhdio.h:23-33)
enum StateSlot { S_RU = 0, S_RV, S_RW, S_TT, S_RO, S_BX, S_BY, S_BZ };
// field slots of the right-hand sides
enum FluxSlot { F_FU = 0, F_FV, F_FW, F_FR, F_FT, F_WW1, F_WW2, F_WW3 };

struct Grid {
    int nx, ny, nz;  // full sizes, ghosts included
    int nPz;
    long long sy, sz;
};

// Scalars of set()/main() (3dmhd.cpp:144-145,354-369,401-459) and device
// pointers to the 1-D metric arrays (3dmhddata.h:21-23).
struct Consts {
    double C13, C23, C43;
    double hx, h2x, hy, h2y, hz, h2z;
    double GRAV, THETA, RE, REPR, ORE, OCV, CV, GAMMA, OMX, OMZ, RM, ORM, OBETA, TB, TP, SFF;
    double DDXmin;  // min of DDX over interior x (NaN skipped), for the CFL reduction
    // Plume terms (3dmhdsub.h:443-459,750-778): pl_mode 0 none, 1 cooling spot
    // on the top wall with iTCon 0, 2 the same with iTCon 1, 3 internal heat
    // sink (iTCon 2).  plx/ply/plz are the host-computed Gaussian factors per
    // x, y, z; pl_tpr (top spot) and pl_s (sink amplitude) depend on TIMT and
    // are refreshed by the host before every step.
    int pl_mode, pl_pad_;
    const double *plx, *ply, *plz;
    double pl_hh, pl_tpr, pl_s;
    // lRem (3dmhdsub.h:229-238,297-313,783-802,852-854): per-substage arrays
    // filled before the right-hand side: lrem_ttm = horizontal mean of T per
    // z, lrem_hrad = HRAD, lrem_g = HRAD minus the z second derivative of the
    // mean (the fused kernels' form); TU, DZTU, DZTB for BCON
    int lrem, lrem_pad_;
    const double *lrem_ttm, *lrem_hrad, *lrem_g;
    double TU, DZTU, DZTB;
    int izCon, iTCon, iBCon, pad_;
    const double *dxxdx, *d2xxdx2, *DDX;
    const double *dyydy, *d2yydy2, *DDY;
    const double *dzzdz, *d2zzdz2, *DDZ;
    const double *RKAPA, *DKAPA;
};

struct Fields8 {
    double* p[8];
};

// Metric coefficients premultiplied for the fused kernels:
//   c1 = duudu*hu, c2a = d2uudu2*hu, c2b = duudu^2*h2u   per axis.
struct Coefs {
    const double *cx1, *cx2a, *cx2b;
    const double *cy1, *cy2a, *cy2b;
    const double *cz1, *cz2a, *cz2b;
    // second-derivative coefficients with the viscous and resistive scales
    // folded in, per axis: ORE*c2a, ORE*c2b, ORE*C43*c2a, ORE*C43*c2b, ORM*c2a, ORM*c2b
    const double* s2[3][6];
    const double *kapz, *dkapz;  // (OCV/REPR)*RKAPA[z], (OCV/REPR)*DKAPA[z]
    const double* dkz;           // dkapz[z] * cz1[z]
    const double* ocz1;          // OBETA * cz1[z]
    // with uniform_xy, per z: kapz*cx2b, kapz*cy2b, then the factors of T(z+1) and T(z-1)
    // kapz*(cz2b + cz2a) + dkapz*cz1 and kapz*(cz2b - cz2a) - dkapz*cz1, and kapz*S_T
    const double* condT[5];
    // per z, for the scale pairs k = 0, 1, 2 (ORE, ORE*C43, ORM) and unscaled (k = 3):
    // lapZ[2k] = b + a, lapZ[2k+1] = b - a of the z second-derivative coefficients
    const double* lapZ[8];
    // uniform x and y grids: d2xxdx2 and d2yydy2 vanish and the x / y
    // coefficients are the same in every interior column
    int uniform_xy;
    // with uniform_xy: the same first-derivative coefficient on x and y
    // (cx1 = cy1, equal spacings), so the x and y advection and induction
    // terms of a component can share one metric product
    int isotropic_xy;
    // with uniform_xy, per z: S = 2 (sx + sy + sz) of the second-derivative
    // coefficients (the 'b' ones) of the Laplacians of u, v, w (viscous,
    // C43 on the x, y, z axis respectively), T (plain), B (resistive), and
    // 2 (sx + sy) of B for the wall planes
    const double* lapS[6];
    // with uniform_xy, per z: the viscous cross-term factors C13*ORE*cx1*cz1 and C13*ORE*cy1*cz1
    const double *kxz, *kyz;
};

// ---- launchers implemented in the .cu files ----------------------------
// Parity path (compiled with -fmad=false, bit-exact with the reference).
int parity_fluxes(unsigned sw, const Grid& g, const Consts& c, Fields8 U, Fields8 F, double* P, double* UU,
                  double* VV, double* WW, cudaStream_t st);
// The same right-hand sides with 1/rho written to RI instead of RO (RO is
// only read); every scratch array is fully written before it is read.
int parity_fluxes_ext(unsigned sw, const Grid& g, const Consts& c, Fields8 U, Fields8 F, double* RI, double* P,
                      double* UU, double* VV, double* WW, cudaStream_t st);
int parity_rk(int kind, int nf, const Grid& g, Fields8 U, Fields8 Z, Fields8 F, double coef, cudaStream_t st);
int parity_bcon(unsigned sw, const Grid& g, const Consts& c, Fields8 U, double timt, cudaStream_t st);
int parity_communicate(int nf, const Grid& g, Fields8 U, cudaStream_t st);
// lRem: horizontal means of T per z (in the reference's summation order when
// `exact`, else by a parallel reduction), then HRAD and the fused form
// G = HRAD - d2(TTM)/dz2, into buf = [TTM | HRAD | G] (3 x nz doubles).
int lrem_profiles(const Grid& g, const Consts& c, const double* TT, double* buf, bool exact, cudaStream_t st);
// HRAD and G from the plane means already in buf[0, nz) (buf as lrem_profiles)
int lrem_hrad_from_means(const Grid& g, const Consts& c, double* buf, cudaStream_t st);
// CFL partial minima/maxima; out[0..4] = UMACH^2-candidate max, w0..w3 minima.
int parity_cfl(bool mag, const Grid& g, const Consts& c, Fields8 U, double* partials, int max_blocks,
               double* out5, cudaStream_t st);
// Conserved totals and max |div B|; out[0..3] = mass, energy, max divB, flags.
int diag_reduce(bool mag, const Grid& g, const Consts& c, Fields8 U, double* partials, int max_blocks, double* out4,
                cudaStream_t st);

// Measured FP64 FMA throughput of the current device (TFLOP/s, 2 flops per FMA).
int fp64_peak(double* tflops);

// Fused FP64 path.
struct FusedArgs {
    Grid g;
    Consts c;
    Coefs k;
    Fields8 U;     // state read (with ghosts)
    Fields8 Uo;    // state written (interior + x/y ghost images)
    Fields8 Z;     // RK register (read when substage > 0, written when substage < 2)
    double* FT;    // persistent temperature right-hand side (lShr only)
    double gdt;    // GAM_k * dt
    double zdt;    // ZETA_k * dt
    double timt;   // simulation time seen by BCON
    int substage;  // 0, 1, 2
    // device-resident time step (adaptive CFL without a host round trip):
    // when dtp is set, gdt = gam * dtp[0] and zdt = zet * dtp[0]
    const double* dtp;
    double gam, zet;
    // interior z planes [zlo, zhi) of a single-instance launch (zhi = 0: all)
    int zlo, zhi;
};
// Device time-step record of mhd_steps_cfl: [0] DT in use (0 once halted),
// [1] TIMT, [2] UMACH, [3] halt flag (DT < 1e-8), [4] the CFL DT computed
// last, [5] completed steps, [6] TIMI, [7] TIMC.
constexpr int kDtRecord = 8;
int cfl_dt_on_device(bool mag, const Grid& g, const Consts& c, Fields8 U, double* partials, int max_blocks,
                     double* rec, cudaStream_t st);
int fused_substage(unsigned sw, const FusedArgs& a, cudaStream_t st);
// the instantiation with the optional temperature terms (fused_substage calls it)
int fused_substage_xp(unsigned sw, const FusedArgs& a, cudaStream_t st);
// Ragged batches: persistent CTAs take (instance, tile x, tile y) items from a
// counter that must be zero at launch.  Tile shapes: 0 = 32x4, 1 = 32x8, 2 = 16x8.
constexpr int kBatchTiles = 3;
void batch_tile_dims(int tile, int* tx, int* ty);
// Per-call control of a ragged batch (device pointers): left[i] = the steps
// instance i still takes in this call (its items are skipped at 0); err[0] =
// the first failed item check (0 = none), err[1..3] = that item (instance,
// tile x | tile y << 16, z range); n = the number of instances.
struct BatchCtl {
    int* left;
    int* err;
    int n;
};

// Check of a work item and of its instance's arguments before a kernel uses
// them: an item that fails records its code in ctl.err and is skipped, so a
// malformed work list shows up as an error status instead of a stray access.
// Codes: 1 instance index, 2 grid sizes, 3 tile position, 4 z range, 5 a
// field pointer is null.
template <class A>
__device__ __forceinline__ bool batch_item_ok(const BatchCtl& ctl, const A* args, int4 it, int tx, int ty, int nf) {
    int code = 0;
    if (it.x < 0 || it.x >= ctl.n) {
        code = 1;
    } else {
        const A& a = args[it.x];
        const int zb = it.w & 0xffff, ze = it.w >> 16;
        if (a.g.nx < 3 || a.g.ny < 3 || a.g.nz < 6 || a.g.sy != a.g.nx || a.g.sz != (long long)a.g.nx * a.g.ny)
            code = 2;
        else if (it.y < 0 || it.z < 0 || 1 + it.y * tx > a.g.nx - 2 || 1 + it.z * ty > a.g.ny - 2)
            code = 3;
        else if (zb < 1 || ze > a.g.nz - 1 || zb >= ze)
            code = 4;
        else
            for (int f = 0; f < nf; f++)
                if (!a.U.p[f] || !a.Uo.p[f] || !a.Z.p[f]) code = 5;
    }
    if (code) {
        if (atomicCAS(ctl.err, 0, code) == 0) {
            ctl.err[1] = it.x;
            ctl.err[2] = it.y | (it.z << 16);
            ctl.err[3] = it.w;
        }
        return false;
    }
    return true;
}

// _uxy: uniform x/y grids (d2xxdx2 = d2yydy2 = 0); _gen: any grid.
// Item w = first z plane | (end plane << 16).
int fused_batch_substage_uxy(unsigned sw, int tile, const FusedArgs* args, const int4* items, int nitems, int* counter,
                             BatchCtl ctl, int grid, cudaStream_t st);
int fused_batch_substage_gen(unsigned sw, int tile, const FusedArgs* args, const int4* items, int nitems, int* counter,
                             BatchCtl ctl, int grid, cudaStream_t st);
int fused_batch_occupancy_uxy(unsigned sw, int tile, int* blocks_per_sm);
int fused_batch_occupancy_gen(unsigned sw, int tile, int* blocks_per_sm);
int fused_batch_bcon(unsigned sw, const FusedArgs* args, const int2* items, BatchCtl ctl, int nblocks,
                     cudaStream_t st);
// end of a batched step: left[i] -= 1 where positive
int batch_tick(int* left, int n, cudaStream_t st);
int fused_bcon_ghost(unsigned sw, const Grid& g, const Consts& c, Fields8 U, double timt, cudaStream_t st);
// BCON of one wall (0 = bottom plane 1, 1 = top plane nz-2) or both (wall = -1)
int fused_bcon_wall(unsigned sw, const Grid& g, const Consts& c, Fields8 U, double timt, int wall, cudaStream_t st);

// FP32-storage path (fields stored in FP32, RO and TT as deviations from FP64
// reference profiles rho0(z), T0(z)).
struct Fields8f {
    float* p[8];
};
// rows of the FP32 kernels' per-z float table (Fused32Args::zf)
constexpr int kZfRows = 12;
struct Fused32Args {
    Grid g;
    Consts c;
    Coefs k;
    Fields8f U;    // state read (deviation form, with ghosts)
    Fields8f Uo;   // state written
    Fields8 Z;     // FP64 RK register (full values)
    double* FT;    // FP64 persistent temperature right-hand side (lShr only)
    const double *bgR, *bgT;     // reference profiles rho0(z), T0(z)
    const double *dzT0, *d2zT0;  // their premultiplied first and second z derivatives
    const float* zf;             // [kZfRows][nz] float cz1, cz2a, cz2b, dzT0, d2zT0, RKAPA, DKAPA, the
                                 // profiles' hydrostatic residual rho0 GRAV - D_z(rho0 T0), and
                                 // rho0, T0 as float pairs (rows 8, 9 and 10, 11: hi, lo)
    double gdt, zdt;
    double timt;
    int substage;
    // device time-step record of mhd_steps_cfl (as FusedArgs)
    const double* dtp;
    double gam, zet;
};
int fused32_substage(unsigned sw, const Fused32Args& a, cudaStream_t st);
int fused32_bcon_ghost(unsigned sw, const Grid& g, const Consts& c, Fields8f U, Fields8 Z, const double* bgR,
                       const double* bgT, double timt, cudaStream_t st);
int communicate32(int nf, const Grid& g, Fields8f U, cudaStream_t st);
// lRem profiles (as lrem_profiles) of an FP32-storage temperature: the plane
// means T0(z) + mean(dT) summed in FP64
int lrem_profiles32(const Grid& g, const Consts& c, const float* dT, const double* bgT, double* buf, cudaStream_t st);
// ragged batches of FP32-storage instances (tile 32x8; same item and counter
// conventions as the FP64 batch)
constexpr int kBatch32TX = 32, kBatch32TY = 8;
int fused32_batch_substage(unsigned sw, const Fused32Args* args, const int4* items, int nitems, int* counter,
                           BatchCtl ctl, int grid, cudaStream_t st);
int fused32_batch_occupancy(unsigned sw, int* blocks_per_sm);
int fused32_batch_bcon(unsigned sw, const Fused32Args* args, const int2* items, BatchCtl ctl, int nblocks,
                       cudaStream_t st);
// CFL reduction of an FP32-storage state (the FP64 row kernel on the widened
// fields): out5 as parity_cfl, or the device time-step record as cfl_dt_on_device
int cfl32_rows(bool mag, const Grid& g, const Consts& c, Fields8f U, const double* bgR, const double* bgT,
               double* partials, int max_blocks, double* out5, cudaStream_t st);
int cfl32_dt_on_device(bool mag, const Grid& g, const Consts& c, Fields8f U, const double* bgR, const double* bgT,
                       double* partials, int max_blocks, double* rec, cudaStream_t st);
int diag32(bool mag, const Grid& g, const Consts& c, Fields8f U, const double* bgR, const double* bgT,
           double* partials, int max_blocks, double* out4, cudaStream_t st);

constexpr unsigned kSwRot = 0x1u, kSwMag = 0x2u, kSwShr = 0x10u;

}  // namespace mhd

// Dispatch a runtime switch word to Switches<MAG,ROT,SHR> template instances.
#define MHD_DISPATCH_SW(sw, FN, ...)                                                  \
    do {                                                                              \
        const bool m_ = ((sw) & ::mhd::kSwMag) != 0;                                  \
        const bool r_ = ((sw) & ::mhd::kSwRot) != 0;                                  \
        const bool s_ = ((sw) & ::mhd::kSwShr) != 0;                                  \
        if (m_ && r_ && s_) FN<::mhd::Switches<true, true, true>>(__VA_ARGS__);       \
        else if (m_ && r_) FN<::mhd::Switches<true, true, false>>(__VA_ARGS__);       \
        else if (m_ && s_) FN<::mhd::Switches<true, false, true>>(__VA_ARGS__);       \
        else if (m_) FN<::mhd::Switches<true, false, false>>(__VA_ARGS__);            \
        else if (r_ && s_) FN<::mhd::Switches<false, true, true>>(__VA_ARGS__);       \
        else if (r_) FN<::mhd::Switches<false, true, false>>(__VA_ARGS__);            \
        else if (s_) FN<::mhd::Switches<false, false, true>>(__VA_ARGS__);            \
        else FN<::mhd::Switches<false, false, false>>(__VA_ARGS__);                   \
    } while (0)
