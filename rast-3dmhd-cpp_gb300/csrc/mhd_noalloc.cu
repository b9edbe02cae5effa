// mhd_noalloc.cu -- mhd_fluxes_noalloc: the right-hand sides of fluxes()
// computed on caller-owned device buffers without allocating anything.
//
// Some callers cannot call cudaMalloc: a service that reserved all of its
// HBM up front in its own pool and hands out slices of it, or a control loop
// that must not hit cudaMalloc's implicit device synchronisation while other
// streams are busy.  This entry point takes every input and output as a
// device pointer the caller already owns; the five scratch fields the
// computation needs (pressure, 1/rho and the three velocities over every
// cell) live in the file-scope device array below instead of in a context.
//
// The array is MHD_NOALLOC_MAX_CELLS * 5 doubles (15.7 MB) and is held by
// every GPU on which this entry point has run, until the process exits.  CUDA
// loads device code lazily, so the first call on a device loads this
// module, reserves the array and looks up its device address with
// cudaGetSymbolAddress (with that device current); callers make that first
// call before their pool takes the rest of the device's memory and before any
// stream capture.  The address is cached per device; it does not survive a
// cudaDeviceReset, after which this entry point must not be used in the
// same process.  The scratch keeps the last
// call's contents: nothing in it has to start at zero, because each call
// writes every scratch cell it later reads.  All calls share this one array,
// so calls whose work overlaps on the GPU (different streams, or different
// host threads) race on it; callers must serialise them.
#include "../../include/mhd_gb300.h"
#include "mhd_common.cuh"

#include <cmath>
#include <cstdio>
#include <mutex>

using namespace mhd;

namespace {

static __device__ __align__(256) double g_noalloc_scratch[(size_t)MHD_NOALLOC_MAX_CELLS * 5];

constexpr int kMaxDevices = 64;
double* g_scratch_addr[kMaxDevices] = {};
std::mutex g_setup_mutex;

// Device address of the scratch array on the current device (set-up, once per device).
int scratch_on_current_device(double** out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return MHD_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            fprintf(stderr, "mhd_fluxes_noalloc: cudaGetSymbolAddress failed: %s\n", cudaGetErrorString(e));
            return MHD_ERR_CUDA;
        }
        g_scratch_addr[dev] = static_cast<double*>(p);
    }
    *out = g_scratch_addr[dev];
    return MHD_OK;
}

}  // namespace

extern "C" int mhd_fluxes_noalloc(const mhd_fluxes_noalloc_args* a, void* stream) {
    if (!a) return MHD_ERR_INVALID;
    const long long nx = a->nPx + 2LL, ny = a->nPy + 2LL, nz = a->nPz + 2LL;
    if (a->nPx < 2 || a->nPy < 2 || a->nPz < 4) {
        fprintf(stderr, "mhd_fluxes_noalloc: need nPx, nPy >= 2 and nPz >= 4\n");
        return MHD_ERR_INVALID;
    }
    if (nx * ny * nz > (long long)MHD_NOALLOC_MAX_CELLS) {
        fprintf(stderr,
                "mhd_fluxes_noalloc: the grid has %lld cells with ghosts, more than the %d cells of the "
                "no-allocation scratch (MHD_NOALLOC_MAX_CELLS); use mhd_create/mhd_fluxes for larger grids\n",
                nx * ny * nz, (int)MHD_NOALLOC_MAX_CELLS);
        return MHD_ERR_INVALID;
    }
    const unsigned sw = a->switches & (MHD_SW_LROT | MHD_SW_LMAG | MHD_SW_LSHR);
    if ((a->switches & MHD_SW_LREM) || (a->izCon != 0 && a->izCon != 1) ||
        (a->iTCon != 0 && a->iTCon != 1 && a->iTCon != 4) || a->iBCon != 0 ||
        ((a->iTCon == 0 || a->iTCon == 1) && a->TP != 0.0))
        return MHD_ERR_UNSUPPORTED;
    const int nf = (sw & MHD_SW_LMAG) ? 8 : 5;
    for (int f = 0; f < nf; f++)
        if (!a->state[f] || !a->flux[f]) return MHD_ERR_INVALID;
    const double* metric[11] = {a->dxxdx, a->d2xxdx2, a->DDX, a->dyydy, a->d2yydy2, a->DDY,
                                a->dzzdz, a->d2zzdz2, a->DDZ, a->RKAPA, a->DKAPA};
    for (const double* m : metric)
        if (!m) return MHD_ERR_INVALID;

    double* scratch = nullptr;
    int rc = scratch_on_current_device(&scratch);
    if (rc) return rc;

    // constants exactly as mhd_create derives them (set(), 3dmhd.cpp:144-145,354-369,432-459)
    mhd_params p = {};
    p.nPx = a->nPx;
    p.nPy = a->nPy;
    p.nPz = a->nPz;
    p.switches = a->switches;
    p.RE = a->RE; p.PR = a->PR; p.RY = a->RY; p.ANG = a->ANG; p.RM = a->RM; p.BETA = a->BETA; p.GAMMA = a->GAMMA;
    mhd_constants k;
    mhd_compute_constants(&p, &k);

    Grid g{};
    g.nx = (int)nx;
    g.ny = (int)ny;
    g.nz = (int)nz;
    g.nPz = a->nPz;
    g.sy = nx;
    g.sz = nx * ny;
    Consts c{};
    c.C13 = k.C13; c.C23 = k.C23; c.C43 = k.C43;
    c.hx = k.hx; c.h2x = k.h2x; c.hy = k.hy; c.h2y = k.h2y; c.hz = k.hz; c.h2z = k.h2z;
    c.GRAV = a->GRAV; c.THETA = a->THETA; c.RE = a->RE; c.REPR = k.REPR; c.ORE = k.ORE; c.OCV = k.OCV; c.CV = k.CV;
    c.GAMMA = a->GAMMA; c.OMX = k.OMX; c.OMZ = k.OMZ; c.RM = a->RM; c.ORM = k.ORM; c.OBETA = k.OBETA;
    c.TB = a->TB; c.TP = a->TP; c.SFF = a->SFF;
    c.DDXmin = -HUGE_VAL;  // no CFL reduction here
    c.izCon = a->izCon; c.iTCon = a->iTCon; c.iBCon = a->iBCon;
    c.dxxdx = a->dxxdx; c.d2xxdx2 = a->d2xxdx2; c.DDX = a->DDX;
    c.dyydy = a->dyydy; c.d2yydy2 = a->d2yydy2; c.DDY = a->DDY;
    c.dzzdz = a->dzzdz; c.d2zzdz2 = a->d2zzdz2; c.DDZ = a->DDZ; c.RKAPA = a->RKAPA; c.DKAPA = a->DKAPA;

    Fields8 U{}, F{};
    for (int f = 0; f < 8; f++) {
        U.p[f] = const_cast<double*>(a->state[f]);  // read only: 1/rho goes to the scratch
        F.p[f] = a->flux[f];
    }
    const size_t n = (size_t)(nx * ny * nz);
    double* P = scratch;
    double* RI = scratch + n;
    double* UU = scratch + 2 * n;
    double* VV = scratch + 3 * n;
    double* WW = scratch + 4 * n;
    const int e = parity_fluxes_ext(sw, g, c, U, F, RI, P, UU, VV, WW, (cudaStream_t)stream);
    return e ? MHD_ERR_CUDA : MHD_OK;
}
