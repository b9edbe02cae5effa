// mhd_io.cu -- state files in the reference's dump layout (host code only).
//
// The reference writes, per MPI rank, "<prefix>.dat0.PPPP" (PPPP = rank,
// 3dmhd.cpp:266,497-502) holding records of RU RV RW TT RO [BX BY BZ]; each
// field is the rank's interior block, x fastest (save(), 3dmhdutils.h:105-110),
// and record idx starts at byte idx * nfields * nCore * 8 (dumpData,
// 3dmhdio.h:20-35).  Ranks are laid out myPEy = rank % nPEy,
// myPEz = rank / nPEy (3dmhd.cpp:95-96) over nRy = nPy/nPEy rows and
// nRz = nPz/nPEz planes.  These functions cut a global state into that layout
// (and back), so a GPU run can restart from a reference dump and the reference
// from a GPU dump.  Unlike the reference's ofstream(binary|ate), writing a
// record keeps the records already in the file.
#include "../../include/mhd_gb300.h"

#include <cstdio>
#include <string>
#include <vector>

namespace {

std::string rank_file(const char* prefix, int rank) {
    char ext[16];
    snprintf(ext, sizeof ext, "%04d", rank);
    return std::string(prefix) + ".dat0." + ext;
}

bool check_layout(int nPx, int nPy, int nPz, int nfields, int nPEy, int nPEz) {
    return nPx >= 1 && nPy >= 1 && nPz >= 1 && (nfields == 5 || nfields == 8) && nPEy >= 1 && nPEz >= 1 &&
           nPy % nPEy == 0 && nPz % nPEz == 0;
}

}  // namespace

extern "C" int mhd_write_dat0(const char* prefix, int nPx, int nPy, int nPz, int nfields, const double* state,
                              int nPEy, int nPEz, int idx) {
    if (!prefix || !state || idx < 0 || !check_layout(nPx, nPy, nPz, nfields, nPEy, nPEz)) return MHD_ERR_INVALID;
    const int nx = nPx + 2, ny = nPy + 2, nz = nPz + 2;
    const int nRy = nPy / nPEy, nRz = nPz / nPEz;
    const size_t nCore = (size_t)nPx * nRy * nRz;
    const size_t ncell = (size_t)nx * ny * nz;
    std::vector<double> buf(nCore);
    for (int rank = 0; rank < nPEy * nPEz; rank++) {
        const int py = rank % nPEy, pz = rank / nPEy;
        const std::string fn = rank_file(prefix, rank);
        FILE* f = fopen(fn.c_str(), "r+b");
        if (!f) f = fopen(fn.c_str(), "w+b");
        if (!f) return MHD_ERR_INVALID;
        const long long off = (long long)idx * nfields * (long long)nCore * 8;
        if (fseeko(f, (off_t)off, SEEK_SET) != 0) {
            fclose(f);
            return MHD_ERR_INVALID;
        }
        for (int fld = 0; fld < nfields; fld++) {
            const double* a = state + (size_t)fld * ncell;
            size_t k = 0;
            for (int z = 1; z <= nRz; z++)
                for (int y = 1; y <= nRy; y++) {
                    const size_t row = ((size_t)(pz * nRz + z) * ny + (size_t)(py * nRy + y)) * nx;
                    for (int x = 1; x <= nPx; x++) buf[k++] = a[row + x];
                }
            if (fwrite(buf.data(), sizeof(double), nCore, f) != nCore) {
                fclose(f);
                return MHD_ERR_INVALID;
            }
        }
        fclose(f);
    }
    return MHD_OK;
}

extern "C" int mhd_read_dat0(const char* prefix, int nPx, int nPy, int nPz, int nfields, double* state, int nPEy,
                             int nPEz, int idx) {
    if (!prefix || !state || idx < 0 || !check_layout(nPx, nPy, nPz, nfields, nPEy, nPEz)) return MHD_ERR_INVALID;
    const int nx = nPx + 2, ny = nPy + 2, nz = nPz + 2;
    const int nRy = nPy / nPEy, nRz = nPz / nPEz;
    const size_t nCore = (size_t)nPx * nRy * nRz;
    const size_t ncell = (size_t)nx * ny * nz;
    std::vector<double> buf(nCore);
    for (int rank = 0; rank < nPEy * nPEz; rank++) {
        const int py = rank % nPEy, pz = rank / nPEy;
        FILE* f = fopen(rank_file(prefix, rank).c_str(), "rb");
        if (!f) return MHD_ERR_INVALID;
        const long long off = (long long)idx * nfields * (long long)nCore * 8;
        if (fseeko(f, (off_t)off, SEEK_SET) != 0) {
            fclose(f);
            return MHD_ERR_INVALID;
        }
        for (int fld = 0; fld < nfields; fld++) {
            if (fread(buf.data(), sizeof(double), nCore, f) != nCore) {
                fclose(f);
                return MHD_ERR_INVALID;
            }
            double* a = state + (size_t)fld * ncell;
            size_t k = 0;
            for (int z = 1; z <= nRz; z++)
                for (int y = 1; y <= nRy; y++) {
                    const size_t row = ((size_t)(pz * nRz + z) * ny + (size_t)(py * nRy + y)) * nx;
                    for (int x = 1; x <= nPx; x++) a[row + x] = buf[k++];
                }
        }
        fclose(f);
    }
    return MHD_OK;
}
