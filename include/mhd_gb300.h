/*
 * mhd_gb300.h -- C ABI of the GB300-native 3dmhd hot path.
 *
 * Drop-in replacement for the reference's per-timestep functions
 * (thu-scc/Rast-3dmhd-cpp).  A driver that today calls
 *     step()        3dmhdsub.h:31      (CFL dt + three RK3 substages)
 *     fluxes()      3dmhdsub.h:18,194  (right-hand sides)
 *     step_block_ZETA0 / ZETA / GAM    3dmhdsub.h:20-22,155-192
 *     BCON()        3dmhdsub.h:19,720  (z-wall conditions)
 *     communicate() 3dmhdmpi.h:11      (ghost exchange)
 * calls the mhd_* function of the same role instead.  Plain C types only.
 *
 * Layout: every field is a host array double[nz][ny][nx] with x fastest
 * and one ghost cell on each side, nx = nPx+2, ny = nPy+2, nz = nPz+2, as
 * the reference's `data` type (3dmhddata.h:8) on one global domain.  z is
 * depth: index 1 is the top wall, nz-2 the bottom wall, 0 and nz-1 the wall
 * ghost planes.
 *
 * Every function returns an int status (MHD_OK = 0, negative on error) and
 * never exits the process (the reference calls exit_err, 3dmhdutils.h:39-43).
 * mhd_last_error() gives the text of the last failure of a context.
 * A context is driven from one host thread; work is queued on the context's
 * CUDA stream and is asynchronous until mhd_sync() or a download.
 */
#ifndef MHD_GB300_H_
#define MHD_GB300_H_

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MHD_ABI_VERSION 1

/* status codes */
#define MHD_OK 0
#define MHD_ERR_INVALID (-1)      /* bad argument or size */
#define MHD_ERR_UNSUPPORTED (-2)  /* switch / boundary combination not built */
#define MHD_ERR_CUDA (-3)         /* CUDA runtime error (text in mhd_last_error) */
#define MHD_ERR_NUMERIC (-4)      /* non-finite or non-positive rho/T seen by a reduction */
#define MHD_ERR_DT_TOO_SMALL (-5) /* CFL dt below 1e-8 (3dmhd.cpp:292-331) */
#define MHD_ERR_NOMEM (-6)        /* device allocation failed */
#define MHD_ERR_TIMEOUT (-7)      /* a bounded device wait gave up */

/* physics switches (3dmhdparam.h:8-17) */
#define MHD_SW_LROT 0x1u
#define MHD_SW_LMAG 0x2u
#define MHD_SW_LPOT 0x4u /* no effect: the reference never reads lPot */
#define MHD_SW_LREM 0x8u /* MHD_ERR_UNSUPPORTED with lShr; fused or parity path, FP64 or FP32 storage */
#define MHD_SW_LSHR 0x10u

/* storage precision of the state */
#define MHD_PREC_FP64 0
#define MHD_PREC_FP32 1 /* fields stored and stenciled in FP32, RK register and EOS in FP64 */

/* kernel path of mhd_step / mhd_steps */
#define MHD_PATH_FUSED 0  /* one fused pass per RK3 substage (FMA contraction on) */
#define MHD_PATH_PARITY 1 /* the unfused sequence below, bit-exact with the reference */

/* field ids: state 0-7 (dump record order, 3dmhdio.h:23-33), right-hand
 * sides 8-15, RK register 16-23 */
enum {
    MHD_RU = 0, MHD_RV, MHD_RW, MHD_TT, MHD_RO, MHD_BX, MHD_BY, MHD_BZ,
    MHD_FU = 8, MHD_FV, MHD_FW, MHD_FR, MHD_FT, MHD_WW1, MHD_WW2, MHD_WW3,
    MHD_ZRU = 16, MHD_ZRV, MHD_ZRW, MHD_ZTT, MHD_ZRO, MHD_ZBX, MHD_ZBY, MHD_ZBZ,
    MHD_NFIELDS = 24
};

/* Run description: sizes, switches (3dmhdparam.h), the par[] run table
 * (3dmhdset.h:7-24) and the metric arrays (3dmhddata.h:21-23, built by
 * x/y/zJacobi, 3dmhdphsic.h:79-156).  Metric pointers are host arrays of
 * nx / ny / nz doubles, copied at mhd_create. */
typedef struct mhd_params {
    int nPx, nPy, nPz;
    unsigned switches;
    int ixCon, iyCon, izCon, iTCon, iBCon;
    int precision;
    int path;
    int reserved_i[5];
    double RE, PR, THETA, GRAV, RY, ANG, RM, BETA, TP, GAMMA, SFF, TB;
    /* with MHD_SW_LREM: the wall values of the static model (Static(),
     * 3dmhdphsic.h:592-594) used by BCON (3dmhdsub.h:783-802,852-854) */
    double TU, DZTU, DZTB;
    double reserved_d[1];
    const double *dxxdx, *d2xxdx2, *DDX;
    const double *dyydy, *d2yydy2, *DDY;
    const double *dzzdz, *d2zzdz2, *DDZ;
    const double *RKAPA, *DKAPA;
} mhd_params;

/* Derived scalars exactly as set() and main() compute them
 * (3dmhd.cpp:144-145,354-369,432-459), single-precision literals included. */
typedef struct mhd_constants {
    double C13, C23, C43, GAM1, GAM2, GAM3, ZETA1, ZETA2;
    double hx, h2x, hy, h2y, hz, h2z;
    double REPR, ORE, ORM, OBETA, OMX, OMZ, CV, OCV;
} mhd_constants;

/* Per-step results and diagnostics (the reference prints DT and UMACH,
 * 3dmhd.cpp:290, 3dmhdio.h:229-239; the conserved totals are new). */
typedef struct mhd_diag {
    double dt;           /* time step used by the last step */
    double umach;        /* max Mach number of the state the CFL step saw */
    double timt;         /* simulation time (TIMT) */
    double total_mass;   /* sum of rho over interior cells x cell volume */
    double total_energy; /* sum of |rho u|^2/(2 rho) + CV rho T + OBETA |B|^2/2, x cell volume */
    double max_divb;     /* max |Dx Bx + Dy By + Dz Bz| over non-wall interior cells */
    long long nit;       /* completed steps (nIt) */
    int flags;           /* bit 0: non-finite value, bit 1: rho <= 0, bit 2: T <= 0 */
    int reserved;
} mhd_diag;

typedef struct mhd_ctx mhd_ctx;

/* ---- lifetime -------------------------------------------------------- */
/* Replaces the static globals of 3dmhd.cpp:29-39 with device buffers owned
 * by the context.  `stream` is a cudaStream_t (NULL: the context creates
 * its own non-blocking stream). */
int mhd_create(const mhd_params* params, void* stream, mhd_ctx** out);
int mhd_destroy(mhd_ctx* ctx);
int mhd_get_constants(const mhd_ctx* ctx, mhd_constants* out);
/* The same derivation without a context or a GPU (host arithmetic only). */
int mhd_compute_constants(const mhd_params* params, mhd_constants* out);
/* Bytes of device memory the context holds. */
int mhd_device_bytes(const mhd_ctx* ctx, size_t* out);
const char* mhd_last_error(const mhd_ctx* ctx);
const char* mhd_status_string(int status);

/* ---- state transfer (dump / restart, 3dmhdio.h:20-72) ----------------- */
/* Copy one whole field (ghosts included) host <-> device.  A download
 * synchronises the context's stream. */
int mhd_upload(mhd_ctx* ctx, int field, const double* host);
int mhd_download(mhd_ctx* ctx, int field, double* host);
/* All nfields state fields (5 without lMag, else 8) from / to one
 * contiguous host block of nfields * nz*ny*nx doubles in field-id order. */
int mhd_upload_state(mhd_ctx* ctx, const double* host);
int mhd_download_state(mhd_ctx* ctx, double* host);
/* Synthetic initial state written on the device, without host arrays
 * (the reference builds its state on the host in Static(),
 * 3dmhdphsic.h:549-763): polytrope T = 1 + THETA z, rho = T^m with
 * m = GRAV/THETA - 1, interior T *= 1 + noise N(0,1) with N from splitmix64 of
 * (seed, interior cell index) through Box-Muller, Bz = bz0 on interior planes,
 * zero momenta (lShr: rho v = +-rho on the walls), periodic x/y ghosts.
 * zcoord: host array of nz depths.  FP64 contexts; blocks until done. */
int mhd_init_polytrope(mhd_ctx* ctx, const double* zcoord, double noise, unsigned long long seed, double bz0);
/* Simulation time and step counter (TIMT, nIt). */
int mhd_set_time(mhd_ctx* ctx, double timt, long long nit);

/* Dump files in the reference's layout (dumpData / loadData, 3dmhdio.h:20-72):
 * for an nPEy x nPEz rank grid, "<prefix>.dat0.PPPP" per rank holds record idx
 * of RU RV RW TT RO [BX BY BZ], each the rank's interior block x fastest.
 * `state` is nfields host arrays of nz*ny*nx doubles in field-id order (as
 * mhd_download_state fills it); reading fills the interior only (call
 * mhd_communicate after uploading).  Writing keeps earlier records of the
 * file, which the reference's writer truncates.  Host code, no GPU needed. */
int mhd_write_dat0(const char* prefix, int nPx, int nPy, int nPz, int nfields, const double* state, int nPEy,
                   int nPEz, int idx);
int mhd_read_dat0(const char* prefix, int nPx, int nPy, int nPz, int nfields, double* state, int nPEy, int nPEz,
                  int idx);

/* ---- unfused parity ABI: one call per reference function ---------------- */
int mhd_fluxes(mhd_ctx* ctx);                   /* fluxes(FORRANGE), 3dmhdsub.h:194-696 */
int mhd_rk_zeta0(mhd_ctx* ctx);                 /* step_block_ZETA0, 3dmhdsub.h:155-166 */
int mhd_rk_zeta(mhd_ctx* ctx, double coef);     /* step_block_ZETA(coef), 3dmhdsub.h:168-179 */
int mhd_rk_gam(mhd_ctx* ctx, double coef);      /* step_block_GAM(coef), 3dmhdsub.h:181-192 */
int mhd_bcon(mhd_ctx* ctx, double timt);        /* BCON(FORRANGE), 3dmhdsub.h:720-873 */
int mhd_communicate(mhd_ctx* ctx);              /* communicate(), 3dmhdmpi.h:11-143 */
/* CFL time step of step() (3dmhdsub.h:36-106); blocks until known. */
int mhd_cfl_dt(mhd_ctx* ctx, double* dt, double* umach);

/* ---- right-hand sides without any allocation ---------------------------- */
/* No counterpart in the reference.  For callers that cannot call cudaMalloc
 * (a service that reserved its HBM up front in its own pool, or a loop that
 * must not hit cudaMalloc's implicit device synchronisation): computes the
 * same right-hand sides as mhd_fluxes, bit for bit, on device buffers the
 * caller owns, and allocates nothing.  Its scratch is a fixed device array
 * of MHD_NOALLOC_MAX_CELLS x 5 doubles (15.7 MB) inside the library, held by
 * every GPU on which the entry point has run, until the process exits; grids
 * with more than MHD_NOALLOC_MAX_CELLS cells (ghosts included) are rejected
 * with MHD_ERR_INVALID and a message on stderr.  CUDA loads the library's
 * device code lazily, so the FIRST call on a device is the one that loads it,
 * reserves the 15.7 MB and looks up the array's address: make that call
 * (any valid grid) before reserving the rest of the device's memory and
 * before any stream capture.  The address is cached per device for the life
 * of the process; after a cudaDeviceReset the cache is stale, so do not use
 * this entry point again in a process that reset its device.  All calls
 * share the array: calls that overlap on the GPU race and must be serialised
 * by the caller.  Inputs are not modified (RO is only read; the reference
 * inverts it in place).  With lShr, flux[MHD_FT - 8] is read and accumulated,
 * as the reference's FT is. */
#define MHD_NOALLOC_MAX_CELLS 393216
typedef struct mhd_fluxes_noalloc_args {
    int nPx, nPy, nPz;
    unsigned switches;
    int izCon, iTCon, iBCon;
    int reserved_i;
    double RE, PR, THETA, GRAV, RY, ANG, RM, BETA, TP, GAMMA, SFF, TB;
    /* device pointers: metric arrays of nx / ny / nz doubles */
    const double *dxxdx, *d2xxdx2, *DDX;
    const double *dyydy, *d2yydy2, *DDY;
    const double *dzzdz, *d2zzdz2, *DDZ;
    const double *RKAPA, *DKAPA;
    /* device pointers, nz*ny*nx doubles each, in field-id order:
     * state RU RV RW TT RO BX BY BZ (ghosts filled), flux FU FV FW FR FT WW1 WW2 WW3;
     * the B fields and WW1..3 may be NULL without lMag */
    const double* state[8];
    double* flux[8];
} mhd_fluxes_noalloc_args;
int mhd_fluxes_noalloc(const mhd_fluxes_noalloc_args* args, void* stream);

/* ---- plume terms ---------------------------------------------------------- */
/* Parameters of the plume terms (3dmhd.cpp:413-426, par[12..15,52,54]): the
 * cooling spot on the top wall (TP != 0 with iTCon 0 or 1,
 * 3dmhdsub.h:750-778) and the internal heat sink of iTCon 2
 * (3dmhdsub.h:443-459), centred at (XP, YP, ZP) with width HH, switched on
 * over TC (and QFH for the sink).  EXX, WYY, ZEE are the coordinates of every
 * x, y, z index (nx, ny, nz entries, ghosts included; host memory, read
 * during the call).  A context whose switches need these terms rejects
 * steps with MHD_ERR_INVALID until this call; the Gaussian factors are
 * computed here, on the host, with the reference's expressions, so the
 * unfused path stays bit-exact with it. */
typedef struct mhd_plume {
    double XP, YP, ZP, HH, TC, QFH;
    const double *EXX, *WYY, *ZEE;
} mhd_plume;
int mhd_set_plume(mhd_ctx* ctx, const mhd_plume* plume);

/* ---- fused time stepping ------------------------------------------------ */
/* One RK3 step, replacing step() (3dmhdsub.h:31-153).  dt > 0: fixed step;
 * dt <= 0: the reference's CFL step (then the call blocks for the dt).
 * `out` (may be NULL) receives dt/umach/timt/nit. */
int mhd_step(mhd_ctx* ctx, double dt, mhd_diag* out);
/* n fixed-dt steps queued without host synchronisation. */
int mhd_steps(mhd_ctx* ctx, int n, double dt);
/* n steps of the reference's run mode, each with its CFL dt (step(),
 * 3dmhdsub.h:36-106, called from the loop of 3dmhd.cpp:271-331).  On the
 * fused paths (FP64 and FP32 storage) the dt is reduced into a
 * device-resident record that the substage kernels read, so the n steps are
 * queued without host round trips and the call blocks once, at the end (the
 * unfused path, and a plume whose strength depends on TIMT, read dt back
 * each step).  dt agrees bit for bit with mhd_cfl_dt.  When a
 * step's dt falls below 1e-8 (the halt of 3dmhd.cpp:292) the state stays as
 * it was before that step and the call returns MHD_ERR_DT_TOO_SMALL
 * (MHD_ERR_NUMERIC for a non-finite dt).  `out` (may be NULL) receives the
 * dt of the last step computed, umach, timt and nit. */
int mhd_steps_cfl(mhd_ctx* ctx, int n, mhd_diag* out);
/* One fixed-dt fused FP64 step from a host state to a host state: `in` is
 * uploaded and the new state is written to `out` (both nf x nz x ny x nx
 * doubles, field-major as in mhd_upload_state; they may be the same buffer;
 * pinned memory (mhd_host_alloc) lets the copies overlap the computation).
 * The interior is cut into z slabs that are uploaded, stepped and downloaded
 * as a dataflow over five streams (uploads, one per RK3 substage, downloads),
 * so the copies hide behind the kernels;
 * the result is bit-identical to mhd_upload_state + mhd_step +
 * mhd_download_state.  in = NULL steps the device state; out = NULL skips the
 * download and the call does not block (then `in` must stay unchanged until
 * mhd_sync).  Replaces the transfers around step() of a host-resident driver;
 * the reference has no counterpart (its state never leaves the host). */
int mhd_step_host(mhd_ctx* ctx, const double* in, double* out, double dt);
/* n fixed-dt steps through host memory: the same as mhd_step_host(ctx, in,
 * out, dt) followed by n-1 calls mhd_step_host(ctx, out, out, dt) (every step
 * uploads its input and downloads its result; bit-identical), but the steps
 * are enqueued back to back, so each step's first slabs overlap the previous
 * step's last slabs and downloads instead of waiting for them.  Blocks until
 * `out` holds the last result (out = NULL: no downloads, steps 1..n-1 start
 * from the device state, and the call does not block). */
int mhd_steps_host(mhd_ctx* ctx, int n, const double* in, double* out, double dt);
/* Mass, energy, max|div B| and sanity flags of the current state (blocks). */
int mhd_diagnostics(mhd_ctx* ctx, mhd_diag* out);
int mhd_sync(mhd_ctx* ctx);

/* The run parameters Static() reads beyond mhd_params (par[8..10],
 * par[18..22], 3dmhd.cpp:409-423) and the rank grid of the run: the Bx layer
 * depends on the z split (nPEz); nPEy only has to divide nPy. */
typedef struct mhd_static_params {
    int nPEy, nPEz;       /* rank grid of the run being started (3dmhdparam.h:18-19) */
    int nTube;            /* flux-tube model of tube() (3dmhdparam.h:124); only 0 */
    int reserved_i;
    double zMax;          /* depth of the box; Static() integrates on z = zz zMax */
    double PZP, SIGMA;    /* conductivity step position and width (0: none) */
    double POLYS;         /* polytropic index of the lower layer */
    double AMPT;          /* temperature (lShr: RV) noise amplitude */
    double AMPB, BFH, BZP;/* lMag: Bx layer amplitude, FWHM, centre */
    const double* ZEE;    /* nPz + 2 z coordinates, ghosts included (length nz) */
    double reserved_d[4];
} mhd_static_params;

/* The reference's fresh-start initial state (Static(), 3dmhdphsic.h:549-763,
 * followed by communicate() as in 3dmhd.cpp:111-142), computed on the host:
 * `state` receives nf x nz x ny x nx doubles, field-major as in
 * mhd_upload_state, bit-identical to the reference run with the same
 * parameters and rank grid.  Uses THETA, GRAV, BETA, the switches and the
 * grid of `p` only (with MHD_SW_LREM also RE and PR); needs no context and
 * no GPU.  With lMag and AMPB = 0 the field is that of tube() with nTube = 0
 * (zero).  With MHD_SW_LREM the background comes from the ODE of
 * getbackground (3dmhdphsic.h:357-362, integrated by ODEINT/RKQC/RK4,
 * 3dmhdphsic.h:409-522) instead of the PZP/SIGMA/POLYS model; MHD_ERR_NUMERIC
 * where the reference aborts there (a level at depth exactly 2, e.g. with
 * zMax = 2: "Stepsize not significant in RKQC").  MHD_ERR_UNSUPPORTED for
 * nTube 1-5, which give the reference no state: 1 and 3 abort in qromb
 * ("Failure in polint", 3dmhdphsic.h:207-208), 2, 4 and 5 do not compile
 * (3dmhdphsic.h:843-844, 951-954, 984). */
int mhd_static_state(const mhd_params* p, const mhd_static_params* s, double* state);
/* The rest of Static()'s lRem set-up (3dmhdphsic.h:565-594, 616-681): the
 * radiative conductivity of every global z plane, rkapa[nz] (RKAPA), its z
 * derivative dkapa[nz] (DKAPA), the wall ghosts repeating the walls, and
 * walls[3] = {TU, DZTU, DZTB}, which the run then passes in mhd_params and as
 * the RKAPA / DKAPA metric arrays.  Bit-identical with the compiled reference;
 * MHD_ERR_NUMERIC where it aborts (as mhd_static_state). */
int mhd_static_lrem_profile(const mhd_params* p, const mhd_static_params* s, double* rkapa, double* dkapa,
                            double* walls);

/* Self-check: the integer-pipe float<->double conversions the FP32-storage
 * kernels use against the hardware conversions, on n test patterns of seed;
 * *mismatches receives the number of differing results (0 expected). */
int mhd_selftest_convert(long long n, unsigned long long seed, long long* mismatches);

/* ---- ragged batches ------------------------------------------------------ */
/* n independent instances (fused-path contexts with one switch set and one
 * precision, any sizes) stepped together: each RK3 substage is one persistent launch over
 * the tiles of all instances, the whole step is a CUDA graph, and the tile
 * shape is picked by timing every candidate on a scratch copy of the batch
 * (cached per batch signature).  No counterpart in the reference, which runs
 * one instance per MPI job.  Results equal each instance stepped alone with
 * the same tile shape, bit for bit.  The batch orders itself after work
 * already queued on the instances' streams, and their later work after it. */
typedef struct mhd_batch mhd_batch;
int mhd_batch_create(mhd_ctx* const* ctxs, const double* dts, int n, void* stream, mhd_batch** out);
int mhd_batch_destroy(mhd_batch* b);
/* tile shape: -1 = autotune on the next step, 0 = 32x4, 1 = 32x8, 2 = 16x8
 * (FP32-storage batches: 32x8, accepted as 0) */
int mhd_batch_set_tile(mhd_batch* b, int tile);
int mhd_batch_tile(const mhd_batch* b, int* tile);
/* longest z range of a work item, in planes (default 64): an instance with
 * more interior planes is split into about equal ranges of at most zmax */
int mhd_batch_set_zrange(mhd_batch* b, int zmax);
int mhd_batch_zrange(const mhd_batch* b, int* zmax);
/* Time every candidate (tile shape x longest z range 64 / 32 / 16) on a
 * scratch copy of the batch and keep the fastest; ms_per_step (may be NULL,
 * 3 entries) gets the best time per step of each tile shape (0 where a shape
 * is not a candidate), chosen the tile shape.  With ms_per_step NULL a
 * result cached for the same batch signature is reused. */
int mhd_batch_autotune(mhd_batch* b, int* chosen, double* ms_per_step);
/* device bytes the autotuner's scratch copy takes while it runs */
int mhd_batch_autotune_bytes(const mhd_batch* b, unsigned long long* bytes);
int mhd_batch_steps(mhd_batch* b, int nsteps);
/* nsteps batched steps in which instance i takes only its first
 * min(nsteps, max_steps[i]) (host array of n counts): an instance that reaches
 * its count drops out of the work list for the rest of the call, so a
 * server's quantum need not shrink to the shortest remaining request. */
int mhd_batch_steps_limited(mhd_batch* b, int nsteps, const int* max_steps);
/* Wait for the batch's queued steps.  The kernels check every work item
 * against its instance's grid before using it; an item that fails is skipped
 * and reported here as MHD_ERR_INVALID (details on stderr). */
int mhd_batch_sync(mhd_batch* b);

/* ---- device selection and timing ---------------------------------------- */
/* Make `device` current for this thread's later mhd_* calls (one process per
 * GPU, e.g. under torchrun). */
int mhd_set_device(int device);
/* CUDA events on the context's stream: start, then stop returns the elapsed
 * milliseconds (waits for the stop event). */
int mhd_timer_start(mhd_ctx* ctx);
int mhd_timer_stop(mhd_ctx* ctx, double* ms);
/* enable != 0: bracket every fused-substage kernel launch with events;
 * mhd_profile_read sums their durations (ms) and counts the launches since
 * the last enable, after waiting for them. */
int mhd_profile(mhd_ctx* ctx, int enable);
int mhd_profile_read(mhd_ctx* ctx, double* substage_ms, long long* launches);

/* FP64 FMA throughput of the current device in TFLOP/s, measured with
 * independent DFMA chains (the roof of the FP64 path on GB300). */
int mhd_fp64_peak(double* tflops);

/* ---- pinned host memory helpers (for callers without a CUDA toolkit) --- */
int mhd_host_alloc(size_t bytes, void** out);
int mhd_host_free(void* p);

#ifdef __cplusplus
}
#endif

#endif
