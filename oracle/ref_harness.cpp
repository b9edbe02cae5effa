/*
 * ref_harness.cpp -- runs the UNMODIFIED reference 3dmhd hot path as a parity
 * oracle.  Test infrastructure only: nothing in the product links this.
 *
 * Built by oracle/refcase.py against the reference sources where they lie
 * (never copied): the reference's 3dmhd.cpp is #included with its main()
 * renamed, and a generated 3dmhdparam.h / 3dmhdset.h pair (grid sizes,
 * switches, run parameters) shadows the reference's own through GCC's "-I-"
 * include-path split.  MPI comes from oracle/mpishim (forked ranks).
 *
 * Input file (written by oracle/refcase.py): a global single-domain state
 * of (nPz+2) x (nPy+2) x (nPx+2) doubles per field, x fastest, plus the 1-D
 * metric arrays and (format version 2) the coordinate arrays EXX, WYY, ZEE.  Each rank takes its slab (3dmhd.cpp:95-96 rank layout),
 * calls communicate() once like main() does (3dmhd.cpp:142), then runs:
 *   mode 0  fluxes() once                              (3dmhdsub.h:194)
 *   mode 1  N fixed-dt RK3 steps: the body of step()    (3dmhdsub.h:116-152)
 *           without its CFL section
 *   mode 2  N calls of the reference step() itself      (3dmhdsub.h:31-153)
 *   mode 3  one RK3 substage                            (3dmhdsub.h:116-124)
 *   mode 4  as mode 1, then the reference's dumpData() writes record 0 of
 *           "<argv[3]>.dat0.PPPP" per rank                (3dmhdio.h:20-35)
 *   mode 5  the fresh-start initial state: Static(), then communicate()
 *           again (3dmhdphsic.h:549-763, 3dmhd.cpp:111-142); the input
 *           state should be zero (Static() leaves some planes of BX as
 *           it finds them)
 * and every rank writes the part of the global arrays it owns into the
 * output file, so the output is the single-domain equivalent state.
 */
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fcntl.h>
#include <fstream>
#include <iostream>
#include <string>
#include <sys/stat.h>
#include <unistd.h>
#include <vector>

#include <mpi.h>

#define main ref_main
#include "3dmhd.cpp"
#undef main

namespace {

constexpr int32_t kMagic = 0x3344484d; /* "MHD3" */

struct InHeader {
    int32_t magic, version, gx, gy, gz, mag, mode, nsteps;
    int32_t pad[8];
    double dt, TB, TIMT0, reserved[13];
};

inline size_t gidx(int z, int y, int x) {
    return ((size_t)z * (size_t)(nPy + iy) + (size_t)y) * (size_t)(nPx + ix) + (size_t)x;
}

void die(const char* msg) {
    fprintf(stderr, "ref_harness: %s\n", msg);
    exit(2);
}

/* Local slab of a global field (ghosts included). */
void load_field(const double* g, data local) {
    for (int z = 0; z < nz; z++)
        for (int y = 0; y < ny; y++)
            for (int x = 0; x < nx; x++) local[z][y][x] = g[gidx(myPEz * nRz + z, myPEy * nRy + y, x)];
}

void load_zarr(const double* g, double* local) {
    for (int z = 0; z < nz; z++) local[z] = g[myPEz * nRz + z];
}

void load_yarr(const double* g, double* local) {
    for (int y = 0; y < ny; y++) local[y] = g[myPEy * nRy + y];
}

/* Write the cells this rank owns: interior, plus the global boundary ghosts. */
void store_field(int fd, size_t field_slot, data local) {
    const size_t nglob = (size_t)(nPz + iz) * (size_t)(nPy + iy) * (size_t)(nPx + ix);
    int zlo = (myPEz == 0) ? 0 : 1, zhi = (myPEz == nPEz - 1) ? nz : nz - 1;
    int ylo = (myPEy == 0) ? 0 : 1, yhi = (myPEy == nPEy - 1) ? ny : ny - 1;
    std::vector<double> row(nx);
    for (int z = zlo; z < zhi; z++)
        for (int y = ylo; y < yhi; y++) {
            for (int x = 0; x < nx; x++) row[x] = local[z][y][x];
            size_t off = (field_slot * nglob + gidx(myPEz * nRz + z, myPEy * nRy + y, 0)) * sizeof(double);
            if (pwrite(fd, row.data(), sizeof(double) * nx, (off_t)off) != (ssize_t)(sizeof(double) * nx))
                die("pwrite failed");
        }
}

void fixed_dt_step() {
    /* Body of step() (3dmhdsub.h:116-152) with DT supplied by the caller. */
    const int zl = iz / 2, zr = nz - iz / 2;
    const int yl = iy / 2, yr = ny - iy / 2;
    const int xl = ix / 2, xr = nx - ix / 2;
    step_block_ZETA0(FORRANGE);
    fluxes(FORRANGE);
    step_block_GAM(GAM1 * DT, FORRANGE);
    BCON(FORRANGE);
    communicate();
    step_block_ZETA(ZETA1 * DT, FORRANGE);
    fluxes(FORRANGE);
    step_block_GAM(GAM2 * DT, FORRANGE);
    BCON(FORRANGE);
    communicate();
    step_block_ZETA(ZETA2 * DT, FORRANGE);
    fluxes(FORRANGE);
    step_block_GAM(GAM3 * DT, FORRANGE);
    BCON(FORRANGE);
    communicate();
    nIt += 1;
    TIMC += DT;
    TIMT = TIMI + TIMC;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 3) die("usage: ref_harness <input.bin> <output.bin>");
    std::vector<char> raw;
    {
        std::ifstream in(argv[1], std::ios::binary);
        if (!in) die("cannot open input");
        raw.assign(std::istreambuf_iterator<char>(in), std::istreambuf_iterator<char>());
    }
    if (raw.size() < sizeof(InHeader)) die("input too short");
    InHeader h;
    memcpy(&h, raw.data(), sizeof(h));
    if (h.magic != kMagic) die("bad magic");
    if (h.gx != nPx || h.gy != nPy || h.gz != nPz) die("grid size of the input does not match the compiled parameters");
    if (h.mag != (lMag ? 1 : 0)) die("lMag of the input does not match the compiled parameters");

    const int gnx = nPx + ix, gny = nPy + iy, gnz = nPz + iz;
    const size_t nglob = (size_t)gnz * gny * gnx;
    const size_t n_metric = 3 * (size_t)gnx + 3 * (size_t)gny + 5 * (size_t)gnz;
    const size_t n_coord = h.version >= 2 ? (size_t)gnx + gny + gnz : 0;
    const size_t need = sizeof(InHeader) + sizeof(double) * (n_metric + 9 * nglob + n_coord);
    if (raw.size() < need) die("input truncated");
    const double* p = reinterpret_cast<const double*>(raw.data() + sizeof(InHeader));
    const double *g_dxxdx = p, *g_d2xxdx2 = p + gnx, *g_DDX = p + 2 * gnx;
    p += 3 * gnx;
    const double *g_dyydy = p, *g_d2yydy2 = p + gny, *g_DDY = p + 2 * gny;
    p += 3 * gny;
    const double *g_dzzdz = p, *g_d2zzdz2 = p + gnz, *g_DDZ = p + 2 * gnz, *g_RKAPA = p + 3 * gnz,
                 *g_DKAPA = p + 4 * gnz;
    p += 5 * gnz;
    const double* g_fields = p; /* RU RV RW TT RO BX BY BZ FT */
    const double* g_coord = p + 9 * nglob; /* EXX WYY ZEE (version >= 2) */

    /* Output: 24 global arrays (state 8, F 8, Z 8) then 16 + nsteps trailer doubles. */
    const int nsteps = h.nsteps > 0 ? h.nsteps : 0;
    const size_t out_bytes = sizeof(double) * (24 * nglob + 16 + (size_t)nsteps);
    {
        int fd = open(argv[2], O_CREAT | O_TRUNC | O_WRONLY, 0644);
        if (fd < 0) die("cannot create output");
        if (ftruncate(fd, (off_t)out_bytes) != 0) die("ftruncate failed");
        close(fd);
    }
    {
        size_t slot = sizeof(double) * (size_t)std::max(nx * ny, nx * nz) + 4096;
        std::string s = std::to_string(slot);
        setenv("MPISHIM_SLOT_BYTES", s.c_str(), 1);
        std::string np = std::to_string(nPE);
        setenv("MPISHIM_NP", np.c_str(), 1);
    }

    int NN;
    MPI_Init(&argc, &argv);
    MPI_Comm_rank(MPI_COMM_WORLD, &myPE);
    MPI_Comm_size(MPI_COMM_WORLD, &NN);
    if (NN != nPE) die("rank count mismatch");
    myPEy = myPE % nPEy;
    myPEz = myPE / nPEy;
    MPISIZE = MPI_DOUBLE_PRECISION;

    set();
    /* Metric arrays of the requested grid replace the ones set() derived (3dmhd.cpp:461-470). */
    for (int x = 0; x < nx; x++) dxxdx[x] = g_dxxdx[x], d2xxdx2[x] = g_d2xxdx2[x], DDX[x] = g_DDX[x];
    load_yarr(g_dyydy, dyydy);
    load_yarr(g_d2yydy2, d2yydy2);
    load_yarr(g_DDY, DDY);
    load_zarr(g_dzzdz, dzzdz);
    load_zarr(g_d2zzdz2, d2zzdz2);
    load_zarr(g_DDZ, DDZ);
    load_zarr(g_RKAPA, RKAPA);
    load_zarr(g_DKAPA, DKAPA);
    if (h.version >= 2) {
        /* coordinates of the requested grid replace set()'s (plume terms, 3dmhdsub.h:443-459,750-778) */
        for (int x = 0; x < nx; x++) EXX[x] = g_coord[x];
        load_yarr(g_coord + gnx, WYY);
        load_zarr(g_coord + gnx + gny, ZEE);
    }

    data* fields_in[9] = {&RU, &RV, &RW, &TT, &RO, &BX, &BY, &BZ, &FT};
    for (int f = 0; f < 9; f++) {
        if (!lMag && f >= 5 && f <= 7) continue;
        load_field(g_fields + (size_t)f * nglob, *fields_in[f]);
    }
    TB = h.TB;
#if lRem
    /* Static() derives these from its model (3dmhdphsic.h:592-594); the input gives them */
    TU = h.reserved[0];
    DZTU = h.reserved[1];
    DZTB = h.reserved[2];
#endif
    TIMI = h.TIMT0;
    TIMC = 0.0;
    TIMT = TIMI;
    DT = h.dt;

    /* 3dmhd.cpp:142-145 */
    communicate();
    CV = 1.0f / (GAMMA - 1.0f);
    OCV = 1.0f / CV;

    std::vector<double> dt_hist;
    const int zl = iz / 2, zr = nz - iz / 2;
    const int yl = iy / 2, yr = ny - iy / 2;
    const int xl = ix / 2, xr = nx - ix / 2;
    auto t0 = std::chrono::steady_clock::now();
    if (h.mode == 0) {
        fluxes(FORRANGE);
    } else if (h.mode == 1) {
        for (int n = 0; n < nsteps; n++) {
            fixed_dt_step();
            dt_hist.push_back(DT);
        }
    } else if (h.mode == 2) {
        for (int n = 0; n < nsteps; n++) {
            step();
            dt_hist.push_back(DT);
        }
    } else if (h.mode == 4) {
        if (argc < 4) die("mode 4 needs a dump prefix");
        for (int n = 0; n < nsteps; n++) {
            fixed_dt_step();
            dt_hist.push_back(DT);
        }
        dumpData(std::string(argv[3]) + ".dat0." + PEextn(), 0);
    } else if (h.mode == 5) {
        /* a fresh start: Static() then communicate(), as main() (3dmhd.cpp:111-142) */
        Static();
        communicate();
#if lRem
        /* Static() also derived the conductivity profile of every plane and the wall
         * values (3dmhdphsic.h:565-594): RKAPA / DKAPA go out in the FU / FV slots,
         * TU / DZTU / DZTB in the trailer */
        for (int z = 0; z < nz; z++)
            for (int y = 0; y < ny; y++)
                for (int x = 0; x < nx; x++) {
                    FU[z][y][x] = RKAPA[z];
                    FV[z][y][x] = DKAPA[z];
                }
#endif
    } else if (h.mode == 3) {
        step_block_ZETA0(FORRANGE);
        fluxes(FORRANGE);
        step_block_GAM(GAM1 * DT, FORRANGE);
        BCON(FORRANGE);
        communicate();
    } else {
        die("unknown mode");
    }
    MPI_Barrier(MPI_COMM_WORLD);
    double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();

    int fd = open(argv[2], O_WRONLY);
    if (fd < 0) die("cannot reopen output");
    data* out_fields[24] = {&RU,  &RV,  &RW,  &TT,  &RO,  &BX,  &BY,  &BZ,  &FU,  &FV,  &FW,  &FR,
                            &FT,  &WW1, &WW2, &WW3, &ZRU, &ZRV, &ZRW, &ZTT, &ZRO, &ZBX, &ZBY, &ZBZ};
    for (int f = 0; f < 24; f++) store_field(fd, (size_t)f, *out_fields[f]);
    if (myPE == 0) {
        std::vector<double> trailer(16 + (size_t)nsteps, 0.0);
        trailer[0] = TIMT;
        trailer[1] = UMACH;
        trailer[2] = secs;
        trailer[3] = (double)nPE;
        trailer[4] = DT;
#if lRem
        trailer[5] = TU;
        trailer[6] = DZTU;
        trailer[7] = DZTB;
#endif
        for (int n = 0; n < nsteps && n < (int)dt_hist.size(); n++) trailer[16 + n] = dt_hist[n];
        off_t off = (off_t)(sizeof(double) * 24 * nglob);
        if (pwrite(fd, trailer.data(), sizeof(double) * trailer.size(), off) != (ssize_t)(sizeof(double) * trailer.size()))
            die("trailer write failed");
    }
    close(fd);
    MPI_Finalize();
    return 0;
}
