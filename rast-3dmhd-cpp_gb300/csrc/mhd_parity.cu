// mhd_parity.cu -- the unfused "parity" kernels.  Built with -fmad=false.
//
// These reproduce the reference CPU code bit for bit: every right-hand-side
// term is evaluated with the reference's association and accumulated into
// its target in the reference's sweep order (3dmhdsub.h:194-696), so the
// per-cell result of this pointwise replay equals the result of the
// reference's ~150 whole-array sweeps.  Intermediates the reference keeps in
// scratch arrays over extended ranges (the derivatives it later
// differentiates again) are recomputed at the neighbouring node from the
// same formula, which gives the same bits.
//
// Operator conventions (3dmhdutils.h:126-239):
//   D1_u F = ((F[u+1]-F[u-1]) * duudu[u]) * hu
//   D2_u F = ((F[u+1]-F[u-1]) * d2uudu2[u]) * hu + (((F[u+1]-2F)+F[u-1]) * duudu^2) * h2u
//   D1_u(F G) = ((F[u+1]G[u+1] - F[u-1]G[u-1]) * duudu[u]) * hu
// the scale factor is applied last; a scale of 1 is the identity and -1 a
// negation.
#include "mhd_common.cuh"
#include "mhd_convert.cuh"

namespace mhd {
namespace {

struct Ix {
    long long i, sy, sz;
    int x, y, z;
};

__device__ __forceinline__ double d1x(const double* F, long long i, int x, const Consts& c) {
    return ((F[i + 1] - F[i - 1]) * c.dxxdx[x]) * c.hx;
}
__device__ __forceinline__ double d1y(const double* F, long long i, long long sy, int y, const Consts& c) {
    return ((F[i + sy] - F[i - sy]) * c.dyydy[y]) * c.hy;
}
__device__ __forceinline__ double d1z(const double* F, long long i, long long sz, int z, const Consts& c) {
    return ((F[i + sz] - F[i - sz]) * c.dzzdz[z]) * c.hz;
}
__device__ __forceinline__ double d2x(const double* F, long long i, int x, const Consts& c) {
    const double du = c.dxxdx[x];
    return ((F[i + 1] - F[i - 1]) * c.d2xxdx2[x]) * c.hx + (((F[i + 1] - 2 * F[i]) + F[i - 1]) * (du * du)) * c.h2x;
}
__device__ __forceinline__ double d2y(const double* F, long long i, long long sy, int y, const Consts& c) {
    const double du = c.dyydy[y];
    return ((F[i + sy] - F[i - sy]) * c.d2yydy2[y]) * c.hy + (((F[i + sy] - 2 * F[i]) + F[i - sy]) * (du * du)) * c.h2y;
}
__device__ __forceinline__ double d2z(const double* F, long long i, long long sz, int z, const Consts& c) {
    const double du = c.dzzdz[z];
    return ((F[i + sz] - F[i - sz]) * c.d2zzdz2[z]) * c.hz + (((F[i + sz] - 2 * F[i]) + F[i - sz]) * (du * du)) * c.h2z;
}
__device__ __forceinline__ double mdx(const double* F, const double* G, long long i, int x, const Consts& c) {
    return ((F[i + 1] * G[i + 1] - F[i - 1] * G[i - 1]) * c.dxxdx[x]) * c.hx;
}
__device__ __forceinline__ double mdy(const double* F, const double* G, long long i, long long sy, int y,
                                      const Consts& c) {
    return ((F[i + sy] * G[i + sy] - F[i - sy] * G[i - sy]) * c.dyydy[y]) * c.hy;
}
__device__ __forceinline__ double mdz(const double* F, const double* G, long long i, long long sz, int z,
                                      const Consts& c) {
    return ((F[i + sz] * G[i + sz] - F[i - sz] * G[i - sz]) * c.dzzdz[z]) * c.hz;
}

// Pressure, gravity, 1/rho in place and the velocities over the extended
// range (3dmhdsub.h:266-268,274-276).
__global__ void k_prep(Grid g, Consts c, Fields8 U, double* FW, double* P, double* UU, double* VV, double* WW) {
    const long long n = (long long)g.nx * g.ny * g.nz;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(i % g.nx);
        const int y = (int)((i / g.nx) % g.ny);
        const int z = (int)(i / g.sz);
        const double ro = U.p[S_RO][i];
        if (x > 0 && x < g.nx - 1 && y > 0 && y < g.ny - 1 && z > 0 && z < g.nz - 1) FW[i] = ro * c.GRAV;
        P[i] = ro * U.p[S_TT][i];
        const double ri = 1.0 / ro;
        U.p[S_RO][i] = ri;
        UU[i] = U.p[S_RU][i] * ri;
        VV[i] = U.p[S_RV][i] * ri;
        WW[i] = U.p[S_RW][i] * ri;
    }
}

// As k_prep, but 1/rho goes to separate scratch and RO is left as it was.
__global__ void k_prep_ext(Grid g, Consts c, Fields8 U, double* RI, double* FW, double* P, double* UU, double* VV,
                           double* WW) {
    const long long n = (long long)g.nx * g.ny * g.nz;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(i % g.nx);
        const int y = (int)((i / g.nx) % g.ny);
        const int z = (int)(i / g.sz);
        const double ro = U.p[S_RO][i];
        if (x > 0 && x < g.nx - 1 && y > 0 && y < g.ny - 1 && z > 0 && z < g.nz - 1) FW[i] = ro * c.GRAV;
        P[i] = ro * U.p[S_TT][i];
        const double ri = 1.0 / ro;
        RI[i] = ri;
        UU[i] = U.p[S_RU][i] * ri;
        VV[i] = U.p[S_RV][i] * ri;
        WW[i] = U.p[S_RW][i] * ri;
    }
}

template <class SW>
__global__ void k_flux(Grid g, Consts c, Fields8 U, Fields8 F, const double* __restrict__ P,
                       const double* __restrict__ UU, const double* __restrict__ VV, const double* __restrict__ WW) {
    const int nPx = g.nx - 2, nPy = g.ny - 2, nPz = g.nz - 2;
    const long long ncell = (long long)nPx * nPy * nPz;
    const long long sy = g.sy, sz = g.sz;
    const int zl = 1, zr = g.nz - 1;
    const double *RU = U.p[S_RU], *RV = U.p[S_RV], *RW = U.p[S_RW], *TT = U.p[S_TT], *RI = U.p[S_RO];
    const double *BX = U.p[S_BX], *BY = U.p[S_BY], *BZ = U.p[S_BZ];
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < ncell;
         t += (long long)gridDim.x * blockDim.x) {
        const int x = 1 + (int)(t % nPx);
        const int y = 1 + (int)((t / nPx) % nPy);
        const int z = 1 + (int)(t / ((long long)nPx * nPy));
        const long long i = z * sz + y * sy + x;

        // continuity, 3dmhdsub.h:204-227
        double fr = -d1x(RU, i, x, c);
        fr -= d1y(RV, i, sy, y, c);
        double w1 = d1z(RW, i, sz, z, c);
        if (z == zl) w1 = (4.0f * RW[i + sz] - RW[i + 2 * sz]) * (c.hz * c.dzzdz[zl]);
        if (z == zr - 1) w1 = (RW[i - 2 * sz] - 4.0f * RW[i - sz]) * (c.hz * c.dzzdz[zr - 1]);
        fr -= w1;

        // pressure and gravity, 3dmhdsub.h:266-272 (F.FW holds RO*GRAV from k_prep)
        double fw = F.p[F_FW][i];
        fw -= d1z(P, i, sz, z, c);
        double fv = -d1y(P, i, sy, y, c);
        double fu = -d1x(P, i, x, c);

        // momentum advection, 3dmhdsub.h:279-289
        fu -= mdx(RU, UU, i, x, c);
        fu -= mdy(RU, VV, i, sy, y, c);
        fu -= mdz(RU, WW, i, sz, z, c);
        fv -= mdx(RV, UU, i, x, c);
        fv -= mdy(RV, VV, i, sy, y, c);
        fv -= mdz(RV, WW, i, sz, z, c);
        fw -= mdx(RW, UU, i, x, c);
        fw -= mdy(RW, VV, i, sy, y, c);
        fw -= mdz(RW, WW, i, sz, z, c);

        const double ri = RI[i], tt = TT[i];
        // temperature advection, 3dmhdsub.h:293-296.  With lShr the reference
        // never re-initialises FT, so it keeps accumulating across calls.
        double ft;
        if constexpr (!SW::lShr) {
            ft = -(d1x(TT, i, x, c) * UU[i]);
            ft -= d1y(TT, i, sy, y, c) * VV[i];
            ft -= d1z(TT, i, sz, z, c) * WW[i];
        } else {
            ft = F.p[F_FT][i];
        }
        double tmp = c.OCV / c.REPR;
        if (c.lrem && !SW::lShr) {
            // lRem: conduction of W = T - TTM(z) plus the mean profile's HRAD,
            // 3dmhdsub.h:297-313 (W at the stencil points as the reference stores it)
            const double* M = c.lrem_ttm;
            const double wc = tt - M[z];
            const double wxp = TT[i + 1] - M[z], wxm = TT[i - 1] - M[z];
            const double wyp = TT[i + sy] - M[z], wym = TT[i - sy] - M[z];
            const double wzp = TT[i + sz] - M[z + 1], wzm = TT[i - sz] - M[z - 1];
            const double dx = c.dxxdx[x], dy = c.dyydy[y], dz = c.dzzdz[z];
            const double d2wx = ((wxp - wxm) * c.d2xxdx2[x]) * c.hx + (((wxp - 2 * wc) + wxm) * (dx * dx)) * c.h2x;
            const double d2wy = ((wyp - wym) * c.d2yydy2[y]) * c.hy + (((wyp - 2 * wc) + wym) * (dy * dy)) * c.h2y;
            const double d2wz = ((wzp - wzm) * c.d2zzdz2[z]) * c.hz + (((wzp - 2 * wc) + wzm) * (dz * dz)) * c.h2z;
            ft += (d2wx * ri) * tmp;
            ft += (d2wy * ri) * tmp;
            ft += (d2wz * ri) * tmp;
            ft += (ri * c.lrem_hrad[z]) * tmp;
        } else {
            // conduction, 3dmhdsub.h:315-319
            ft += ((d2x(TT, i, x, c) * ri) * c.RKAPA[z]) * tmp;
            ft += ((d2y(TT, i, sy, y, c) * ri) * c.RKAPA[z]) * tmp;
            ft += ((d2z(TT, i, sz, z, c) * ri) * c.RKAPA[z]) * tmp;
            ft += ((d1z(TT, i, sz, z, c) * ri) * c.DKAPA[z]) * tmp;
        }
        // internal plume heat sink (iTCon 2), 3dmhdsub.h:443-459
        if (c.pl_mode == 3) ft -= (((c.pl_s * ri) * c.plx[x]) * c.ply[y]) * c.plz[z];

        // viscous Laplacians, 3dmhdsub.h:462-472
        fu += d2x(UU, i, x, c) * (c.ORE * c.C43);
        fu += d2y(UU, i, sy, y, c) * c.ORE;
        fu += d2z(UU, i, sz, z, c) * c.ORE;
        fv += d2x(VV, i, x, c) * c.ORE;
        fv += d2y(VV, i, sy, y, c) * (c.ORE * c.C43);
        fv += d2z(VV, i, sz, z, c) * c.ORE;
        fw += d2x(WW, i, x, c) * c.ORE;
        fw += d2y(WW, i, sy, y, c) * c.ORE;
        fw += d2z(WW, i, sz, z, c) * (c.ORE * c.C43);

        // viscous cross terms, heating and pdV work, 3dmhdsub.h:475-538
        const double c13ore = c.C13 * c.ORE;
        const double ux = d1x(UU, i, x, c);  // WW1 of do 650
        const double vx = d1x(VV, i, x, c);  // WW2 of do 670
        double vy = 0.0;
        if constexpr (!SW::lShr) {
            const double wx = d1x(WW, i, x, c);  // do 690
            tmp = c.OCV * c.ORE;
            ft += ((ri * ux) * ux) * (tmp * c.C43);
            ft += ((ri * vx) * vx) * tmp;
            ft += ((ri * wx) * wx) * tmp;
            ft -= (ux * tt) * c.OCV;
        }
        fu += (((d1x(VV, i + sy, x, c) - d1x(VV, i - sy, x, c)) * c.dyydy[y]) * c.hy) * c13ore;  // do 720
        fv += (((d1x(UU, i + sy, x, c) - d1x(UU, i - sy, x, c)) * c.dyydy[y]) * c.hy) * c13ore;  // do 730
        if constexpr (!SW::lShr) {
            const double uy = d1y(UU, i, sy, y, c);  // do 740
            tmp = c.OCV * c.ORE;
            ft += ((ri * uy) * uy) * tmp;
            ft += ((ri * uy) * vx) * (tmp * 2);
            vy = d1y(VV, i, sy, y, c);  // do 755
            tmp = c.C43 * c.OCV * c.ORE;
            ft += ((ri * vy) * vy) * tmp;
            ft -= (vy * tt) * c.OCV;
        }
        const double wz = d1z(WW, i, sz, z, c);  // do 790
        if constexpr (!SW::lShr) {
            tmp = c.C43 * c.OCV * c.ORE;
            ft += ((ri * wz) * wz) * tmp;
            ft += ((ri * ux) * wz) * (-tmp);
            ft += ((ri * ux) * vy) * (-tmp);
            ft += ((ri * vy) * wz) * (-tmp);
            ft -= (wz * tt) * c.OCV;
        }
        fu += (((d1z(WW, i + 1, sz, z, c) - d1z(WW, i - 1, sz, z, c)) * c.dxxdx[x]) * c.hx) * c13ore;   // do 840
        fv += (((d1z(WW, i + sy, sz, z, c) - d1z(WW, i - sy, sz, z, c)) * c.dyydy[y]) * c.hy) * c13ore; // do 850
        const double uz = d1z(UU, i, sz, z, c);  // do 860
        const double vz = d1z(VV, i, sz, z, c);  // do 880
        if constexpr (!SW::lShr) {
            const double wy = d1y(WW, i, sy, y, c);  // do 900
            tmp = c.OCV * c.ORE;
            ft += ((ri * uz) * uz) * tmp;
            ft += ((ri * vz) * vz) * tmp;
            ft += ((ri * wy) * wy) * tmp;
            ft += ((ri * vz) * wy) * (2.0f * tmp);
        }
        fw += (((d1z(UU, i + 1, sz, z, c) - d1z(UU, i - 1, sz, z, c)) * c.dxxdx[x]) * c.hx) * c13ore;   // do 920.1
        fw += (((d1z(VV, i + sy, sz, z, c) - d1z(VV, i - sy, sz, z, c)) * c.dyydy[y]) * c.hy) * c13ore; // do 920.2
        if constexpr (!SW::lShr) {
            const double wx = d1x(WW, i, x, c);  // do 930
            tmp = c.OCV * c.ORE;
            ft += ((ri * uz) * wx) * (2.0f * tmp);
        }

        // Coriolis, 3dmhdsub.h:540-545
        if constexpr (SW::lRot) {
            fu += RV[i] * c.OMZ;
            fv -= RU[i] * c.OMZ;
            fv += RW[i] * c.OMX;
            fw -= RV[i] * c.OMX;
        }

        // induction, Lorentz force and Ohmic heating, 3dmhdsub.h:547-695.
        // sRU..sTT stand for the reference's reuse of RU, RV, RW, TT as scratch.
        if constexpr (SW::lMag) {
            const double c1 = c.OBETA * c.ORM * c.OCV;
            const double c2 = -2.0f * c.OBETA * c.ORM * c.OCV;
            const double bx = BX[i], by = BY[i], bz = BZ[i];
            const double u = UU[i], v = VV[i], w = WW[i];
            double sRU = d1x(UU, i, x, c), sRV = d1x(VV, i, x, c), sRW = d1x(WW, i, x, c), sTT;
            double ww2 = bx * sRV;
            ww2 -= by * sRU;
            double ww3 = bx * sRW;
            ww3 -= bz * sRU;
            sRU = d1y(UU, i, sy, y, c);
            sRV = d1y(VV, i, sy, y, c);
            sRW = d1y(WW, i, sy, y, c);
            double ww1 = by * sRU;
            ww1 -= bx * sRV;
            ww3 += by * sRW;
            ww3 -= bz * sRV;
            sRU = d1z(UU, i, sz, z, c);
            sRV = d1z(VV, i, sz, z, c);
            sRW = d1z(WW, i, sz, z, c);
            if (z == zl) sRW = (4.0f * WW[i + sz] - WW[i + 2 * sz]) * c.hz * c.dzzdz[zl];
            if (z == zr - 1) sRW = (-4.0f * WW[i - sz] + WW[i - 2 * sz]) * c.hz * c.dzzdz[zr - 1];
            ww1 += bz * sRU;
            ww1 -= bx * sRW;
            ww2 += bz * sRV;
            ww2 -= by * sRW;
            sRU = d1x(BX, i, x, c);
            sRV = d1x(BY, i, x, c);
            sRW = d1x(BZ, i, x, c);
            sTT = d1y(BX, i, sy, y, c);
            fu += (by * sTT) * c.OBETA;
            fu -= (by * sRV) * c.OBETA;
            fu -= (bz * sRW) * c.OBETA;
            fv += (bx * sRV) * c.OBETA;
            fv -= (bx * sTT) * c.OBETA;
            fw += (bx * sRW) * c.OBETA;
            ft += ((ri * sTT) * sTT) * c1;
            ft += ((ri * sRV) * sRV) * c1;
            ft += ((ri * sRW) * sRW) * c1;
            ft += ((ri * sRV) * sTT) * c2;
            ww1 -= u * sRU;
            ww1 -= v * sTT;
            ww2 -= u * sRV;
            ww3 -= u * sRW;
            sRU = d2x(BX, i, x, c);
            sRV = d2x(BY, i, x, c);
            sTT = d2y(BX, i, sy, y, c);
            ww1 += sRU * c.ORM;
            ww1 += sTT * c.ORM;
            ww2 += sRV * c.ORM;
            sTT = d2x(BZ, i, x, c);
            ww3 += sTT * c.ORM;
            sRU = d1z(BX, i, sz, z, c);
            sRV = d1y(BY, i, sy, y, c);
            fu += (bz * sRU) * c.OBETA;
            fw -= (bx * sRU) * c.OBETA;
            ft += ((ri * sRU) * sRU) * c1;
            ft += ((ri * sRU) * sRW) * c2;
            ww1 -= w * sRU;
            ww2 -= v * sRV;
            sRU = d2z(BX, i, sz, z, c);
            if (z == zl)
                sRU = (-3.0f * BX[i] + 4.0f * BX[i + sz] - BX[i + 2 * sz]) * c.hz * c.d2zzdz2[zl] +
                      (2.0f * BX[i] - 5.0f * BX[i + sz] + 4.0f * BX[i + 2 * sz] - BX[i + 3 * sz]) * c.h2z * c.dzzdz[zl] *
                          c.dzzdz[zl];
            if (z == zr - 1)
                sRU = (3.0f * BX[i] - 4.0f * BX[i - sz] + BX[i - 2 * sz]) * c.hz * c.d2zzdz2[zr - 1] +
                      (2.0f * BX[i] - 5.0f * BX[i - sz] + 4.0f * BX[i - 2 * sz] - BX[i - 3 * sz]) * c.h2z *
                          c.dzzdz[zr - 1] * c.dzzdz[zr - 1];
            sRV = d2y(BY, i, sy, y, c);
            ww1 += sRU * c.ORM;
            ww2 += sRV * c.ORM;
            sRV = d1z(BY, i, sz, z, c);
            sRW = d1y(BZ, i, sy, y, c);
            sRU = sRV;
            sRU -= sRW;
            fv += (bz * sRU) * c.OBETA;
            fw -= (by * sRU) * c.OBETA;
            ft += ((ri * sRV) * sRV) * c1;
            ft += ((ri * sRW) * sRW) * c1;
            ft += ((ri * sRV) * sRW) * c2;
            ww2 -= w * sRV;
            ww3 -= v * sRW;
            sRV = d2z(BY, i, sz, z, c);
            if (z == zl)
                sRV = (-3.0f * BY[i] + 4.0f * BY[i + sz] - BY[i + 2 * sz]) * c.hz * c.d2zzdz2[zl] +
                      (2.0f * BY[i] - 5.0f * BY[i + sz] + 4.0f * BY[i + 2 * sz] - BY[i + 3 * sz]) * c.h2z * c.dzzdz[zl] *
                          c.dzzdz[zl];
            if (z == zr - 1)
                sRV = (3.0f * BY[i] - 4.0f * BY[i - sz] + BY[i - 2 * sz]) * c.hz * c.d2zzdz2[zr - 1] +
                      (2.0f * BY[i] - 5.0f * BY[i - sz] + 4.0f * BY[i - 2 * sz] - BY[i - 3 * sz]) * c.h2z *
                          c.dzzdz[zr - 1] * c.dzzdz[zr - 1];
            sRW = d2y(BZ, i, sy, y, c);
            ww2 += sRV * c.ORM;
            ww3 += sRW * c.ORM;
            sRW = d1z(BZ, i, sz, z, c);
            ww3 -= w * sRW;
            sRW = d2z(BZ, i, sz, z, c);
            ww3 += sRW * c.ORM;
            F.p[F_WW1][i] = ww1;
            F.p[F_WW2][i] = ww2;
            F.p[F_WW3][i] = ww3;
        }
        F.p[F_FU][i] = fu;
        F.p[F_FV][i] = fv;
        F.p[F_FW][i] = fw;
        F.p[F_FR][i] = fr;
        F.p[F_FT][i] = ft;
    }
}

// step_block_ZETA0 / ZETA / GAM over the interior, scale_add = src1 + scale*srcd1
// (3dmhdsub.h:155-192, 3dmhdutils.h:57-59).  kind 0: Z=U, 1: Z=U+c*F, 2: U=Z+c*F.
__constant__ int kFluxOfState[8] = {F_FU, F_FV, F_FW, F_FT, F_FR, F_WW1, F_WW2, F_WW3};

__global__ void k_rk(int kind, int nf, Grid g, Fields8 U, Fields8 Z, Fields8 F, double coef) {
    const int nPx = g.nx - 2, nPy = g.ny - 2, nPz = g.nz - 2;
    const long long ncell = (long long)nPx * nPy * nPz;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < ncell;
         t += (long long)gridDim.x * blockDim.x) {
        const int x = 1 + (int)(t % nPx);
        const int y = 1 + (int)((t / nPx) % nPy);
        const int z = 1 + (int)(t / ((long long)nPx * nPy));
        const long long i = z * g.sz + y * g.sy + x;
        for (int f = 0; f < nf; f++) {
            if (kind == 0) Z.p[f][i] = U.p[f][i];
            else if (kind == 1) Z.p[f][i] = U.p[f][i] + coef * F.p[kFluxOfState[f]][i];
            else U.p[f][i] = Z.p[f][i] + coef * F.p[kFluxOfState[f]][i];
        }
    }
}

// BCON, 3dmhdsub.h:720-873.  One thread per (y, x) of the interior does the
// top wall (z = 1, rank row myPEz == 0 in the reference) and the bottom wall
// (z = nz-2, myPEz == nPEz-1).
template <class SW>
__global__ void k_bcon(Grid g, Consts c, Fields8 U, double timt) {
    const int nPx = g.nx - 2, nPy = g.ny - 2;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nPx * nPy) return;
    const int x = 1 + t % nPx, y = 1 + t / nPx;
    const long long sz = g.sz;
    double *RU = U.p[S_RU], *RV = U.p[S_RV], *RW = U.p[S_RW], *TT = U.p[S_TT], *RO = U.p[S_RO], *BZ = U.p[S_BZ];
    const double RRT = 1.0f, RRB = -1.0f, RPP = 0.0f;
    const int zl = 1, zr = g.nz - 1;
    // top
    long long i = zl * sz + y * g.sy + x;
    if constexpr (SW::lShr) {
        RU[i] = 0.0f;
        RV[i] = RRT * cos(RPP * timt) * RO[i];
    } else {
        RU[i] = RO[i] * (c.C43 * RU[i + sz] / RO[i + sz] - c.C13 * RU[i + 2 * sz] / RO[i + 2 * sz]);
        RV[i] = RO[i] * (c.C43 * RV[i + sz] / RO[i + sz] - c.C13 * RV[i + 2 * sz] / RO[i + 2 * sz]);
    }
    RW[i] = 0.0f;
    if (c.pl_mode == 1) {
        // cooling spot on the top wall, 3dmhdsub.h:750-766
        TT[i] = 1.0f - (1.0f - c.pl_tpr) * c.plx[x] / c.pl_hh * c.ply[y] / c.pl_hh;
    } else if (c.pl_mode == 2) {
        // the same with the fixed-flux wall, 3dmhdsub.h:767-777 (DZ in double here)
        const double DZ = 1.0f / (double)(g.nPz - 1) / c.dzzdz[zl];
        TT[i] = c.C43 * TT[i + sz] - c.C13 * TT[i + 2 * sz] -
                c.C23 * DZ * (c.THETA - (c.THETA - c.pl_tpr) * c.plx[x] / c.pl_hh * c.ply[y] / c.pl_hh);
    } else if (c.iTCon == 1) {
        const double DZ = 1.0f / (float)(g.nPz - 1) / c.dzzdz[zl];
        if (c.lrem) TT[i] = c.C43 * TT[i + sz] - c.C13 * TT[i + 2 * sz] + c.DZTU;  // 3dmhdsub.h:800-802
        else TT[i] = c.C43 * TT[i + sz] - c.C13 * TT[i + 2 * sz] - c.C23 * DZ * c.THETA;
    } else if (c.lrem) {
        TT[i] = c.TU;  // 3dmhdsub.h:783-784
    } else {
        TT[i] = 1.0f;
        if (c.iTCon == 4 && x < g.nx / 2) TT[i] = 1.0f - c.TP;
    }
    if constexpr (SW::lMag) {
        if (c.iBCon == 0) BZ[i] = 0.0f;
    }
    // bottom
    i = (zr - 1) * sz + y * g.sy + x;
    if constexpr (SW::lShr) {
        RU[i] = 0.0f;
        RV[i] = RRB * cos(RPP * timt) * RO[i];
    } else {
        RU[i] = RO[i] * (c.C43 * RU[i - sz] / RO[i - sz] - c.C13 * RU[i - 2 * sz] / RO[i - 2 * sz]);
        RV[i] = RO[i] * (c.C43 * RV[i - sz] / RO[i - sz] - c.C13 * RV[i - 2 * sz] / RO[i - 2 * sz]);
    }
    RW[i] = 0.0f;
    if (c.izCon == 0) {
        TT[i] = c.TB;
    } else if (c.lrem) {
        TT[i] = c.C43 * TT[i - sz] - c.C13 * TT[i - 2 * sz] + c.DZTB;  // 3dmhdsub.h:852-854
    } else {
        const double DZ = 1.0f / (float)(g.nPz - 1) / c.dzzdz[zr - 1];
        TT[i] = c.C43 * TT[i - sz] - c.C13 * TT[i - 2 * sz] - c.C23 * DZ * c.THETA / c.RKAPA[zr - 1];
    }
    if constexpr (SW::lMag) {
        if (c.iBCon == 0) BZ[i] = 0.0f;
    }
}

// communicate(), 3dmhdmpi.h:11-143, on one domain: each x/y ghost cell of
// every plane (wall ghost planes included) takes the value of its periodic
// image V[z][wrap(y)][wrap(x)], wrap(0) = n-2, wrap(n-1) = 1.  Sources are
// never ghosts, so one pass has no ordering hazard.
__global__ void k_comm(int nf, Grid g, Fields8 U) {
    const long long per_plane = 2LL * g.nx + 2LL * (g.ny - 2);
    const long long n = per_plane * g.nz;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x) {
        const int z = (int)(t / per_plane);
        long long r = t % per_plane;
        int y, x;
        if (r < g.nx) {
            y = 0;
            x = (int)r;
        } else if (r < 2LL * g.nx) {
            y = g.ny - 1;
            x = (int)(r - g.nx);
        } else {
            r -= 2LL * g.nx;
            y = 1 + (int)(r / 2);
            x = (r % 2) ? g.nx - 1 : 0;
        }
        const int ys = (y == 0) ? g.ny - 2 : (y == g.ny - 1 ? 1 : y);
        const int xs = (x == 0) ? g.nx - 2 : (x == g.nx - 1 ? 1 : x);
        const long long d = z * g.sz + y * g.sy + x, s = z * g.sz + ys * g.sy + xs;
        for (int f = 0; f < nf; f++) U.p[f][d] = U.p[f][s];
    }
}

// ---- CFL time step of step() (3dmhdsub.h:36-106) ---------------------------
// Per cell: UMACH^2 candidate mc = OGAMMA*UU/T, and four time-step candidates
// a0 = DD/sqrt(UU') (fast mode), a1 (conduction), a2 (viscosity), a3
// (resistivity), with DD the smallest grid spacing at the cell.  The helpers
// keep the reference's expressions and association (this file is compiled
// without FMA contraction), so every candidate is bit-exact.

__device__ __forceinline__ double cfl_dd_yz(const Consts& c, int y, int z) {
    return (c.DDZ[z] < c.DDY[y]) ? c.DDZ[z] : c.DDY[y];
}
__device__ __forceinline__ double cfl_kappa(const Consts& c, int z) {
    return c.lrem ? 1.0f + c.RKAPA[z] : c.RKAPA[z];  // 3dmhdsub.h:79-83
}
__device__ __forceinline__ double cfl_a1(const Consts& c, double DD, double ro, int z) {
    return 0.5f * DD * DD * c.REPR * c.CV * ro / cfl_kappa(c, z);
}
__device__ __forceinline__ double cfl_a2(const Consts& c, double DD, double ro) { return 0.375f * DD * DD * c.RE * ro; }
__device__ __forceinline__ double cfl_a3(const Consts& c, double DD) { return 0.5f * DD * DD * c.RM; }

// float value of d with its significand truncated to 23 bits (relative error
// below 2^-23), formed with integer operations only; magnitudes below 2^-126
// become 0 and magnitudes beyond the float range (and NaN) become infinity.
__device__ __forceinline__ float trunc_to_f32(double d) {
    const unsigned hi = (unsigned)__double2hiint(d), lo = (unsigned)__double2loint(d);
    const unsigned sign = hi & 0x80000000u;
    const int e = (int)((hi >> 20) & 0x7ffu) - (1023 - 127);
    unsigned b;
    if (e <= 0) b = sign;
    else if (e >= 255) b = sign | 0x7f800000u;
    else b = sign | ((unsigned)e << 23) | ((hi & 0x000fffffu) << 3) | (lo >> 29);
    return __uint_as_float(b);
}

__device__ __forceinline__ bool nonzero_bits(double d) {
    return (((unsigned)__double2hiint(d) & 0x7fffffffu) | (unsigned)__double2loint(d)) != 0u;
}

// Field access of the CFL reduction: FP64 state, or FP32-storage state
// (deviations from the FP64 profiles rho0(z), T0(z)) widened to FP64.
struct CflFields64 {
    Fields8 U;
    __device__ double f(int k, long long i) const { return U.p[k][i]; }
    __device__ double ro(long long i, int) const { return U.p[S_RO][i]; }
    __device__ double tt(long long i, int) const { return U.p[S_TT][i]; }
    // the estimate's float input of field k (truncated to 23 bits) and whether it is nonzero
    __device__ float fe(int k, long long i) const { return trunc_to_f32(U.p[k][i]); }
    __device__ bool nz(int k, long long i) const { return nonzero_bits(U.p[k][i]); }
    // Estimate inputs ro, tt of a filtered row (truncated to 23 bits: relative
    // error below 2^-23) and m, the value whose row minimum gives the row's
    // smallest ro: here ro itself.
    struct Row {};
    using Min = double;
    __device__ Row row(int) const { return {}; }
    __device__ void est_in(const Row&, long long i, float& ro, float& tt, bool& ok, double& m) const {
        m = U.p[S_RO][i];
        ro = trunc_to_f32(m);
        tt = trunc_to_f32(U.p[S_TT][i]);
        ok = true;
    }
    __device__ double ro_min(double m, int) const { return m; }
};
struct CflFields32 {
    Fields8f U;
    const double *bgR, *bgT;
    __device__ double f(int k, long long i) const { return widen_f32(U.p[k][i]); }
    __device__ double ro(long long i, int z) const { return bgR[z] + widen_f32(U.p[S_RO][i]); }
    __device__ double tt(long long i, int z) const { return bgT[z] + widen_f32(U.p[S_TT][i]); }
    // stored floats are their own estimate input (exact; subnormals kept)
    __device__ float fe(int k, long long i) const { return U.p[k][i]; }
    __device__ bool nz(int k, long long i) const { return (__float_as_uint(U.p[k][i]) & 0x7fffffffu) != 0u; }
    // Estimate inputs of a filtered row, with no FP64 operation per cell:
    // ro = float(rho0) + dro and tt = float(T0) + dT in FP32.  Against the FP64
    // values their relative error is at most 5 * 2^-24 (the profile's rounding,
    // amplified at most 4 times by cancellation, plus the sum's own), which
    // `ok` requires by |float(rho0)| <= 4 |ro| and |float(T0)| <= 4 |tt|.
    // m = dro: rho0 + dro rounds monotonically in dro, so the row's smallest
    // ro is rho0 plus its smallest dro, one FP64 sum per row.
    struct Row {
        float Rf, Tf;
    };
    using Min = float;
    __device__ Row row(int z) const { return {narrow_f64(bgR[z]), narrow_f64(bgT[z])}; }
    __device__ void est_in(const Row& r, long long i, float& ro, float& tt, bool& ok, float& m) const {
        m = U.p[S_RO][i];
        ro = __fadd_rn(r.Rf, m);
        tt = __fadd_rn(r.Tf, U.p[S_TT][i]);
        ok = fabsf(r.Rf) <= 4.0f * fabsf(ro) && fabsf(r.Tf) <= 4.0f * fabsf(tt);
    }
    __device__ double ro_min(float m, int z) const { return bgR[z] + widen_f32(m); }
};

// mc and the fast-mode speed^2 UU' of cell i (plane z)
template <bool MAG, class FA>
__device__ __forceinline__ void cfl_speeds(const Consts& c, const FA& U, long long i, int z, double OGAMMA, double& mc,
                                           double& uu) {
    const double ru = U.f(S_RU, i), rv = U.f(S_RV, i), rw = U.f(S_RW, i), ro = U.ro(i, z), tt = U.tt(i, z);
    double UU = (ru * ru + rv * rv + rw * rw) / (ro * ro);
    mc = OGAMMA * UU / tt;
    if constexpr (MAG) {
        const double bx = U.f(S_BX, i), by = U.f(S_BY, i), bz = U.f(S_BZ, i);
        UU += c.GAMMA * tt + (bx * bx + by * by + bz * bz) * c.OBETA / ro +
              2.0f * sqrt(UU * (c.GAMMA * tt + (bx * bx + by * by + bz * bz) * c.OBETA / ro));
    } else {
        UU += c.GAMMA * tt + 2.0f * sqrt(c.GAMMA * UU * tt);
    }
    uu = UU;
}

// all five candidates of cell (x, y, z), folded into the running extrema
template <bool MAG, class FA>
__device__ __forceinline__ void cfl_cell(const Grid& g, const Consts& c, const FA& U, int x, int y, int z,
                                         double OGAMMA, double& um, double& w0, double& w1, double& w2, double& w3) {
    const long long i = (long long)z * g.sz + (long long)y * g.sy + x;
    double mc, UU;
    cfl_speeds<MAG>(c, U, i, z, OGAMMA, mc, UU);
    um = (um < mc) ? mc : um;
    double DD = cfl_dd_yz(c, y, z);
    if (g.nx > 3) DD = (c.DDX[x] < DD) ? c.DDX[x] : DD;
    const double ro = U.ro(i, z);
    const double a0 = DD / sqrt(UU);
    const double a1 = cfl_a1(c, DD, ro, z);
    const double a2 = cfl_a2(c, DD, ro);
    w0 = (a0 < w0) ? a0 : w0;
    w1 = (a1 < w1) ? a1 : w1;
    w2 = (a2 < w2) ? a2 : w2;
    if constexpr (MAG) {
        const double a3 = cfl_a3(c, DD);
        w3 = (a3 < w3) ? a3 : w3;
    }
}

// Block reduction of the running extrema into partials [5][gridDim.x]
// (blockDim.x = 256); min/max are exact, so no order changes the result.
__device__ void write_cfl_partials(double um, double w0, double w1, double w2, double w3, double* part) {
    __shared__ double s[5][256];
    s[0][threadIdx.x] = um;
    s[1][threadIdx.x] = w0;
    s[2][threadIdx.x] = w1;
    s[3][threadIdx.x] = w2;
    s[4][threadIdx.x] = w3;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h) {
            const double a = s[0][threadIdx.x + h];
            s[0][threadIdx.x] = (s[0][threadIdx.x] < a) ? a : s[0][threadIdx.x];
            for (int k = 1; k < 5; k++) {
                const double b = s[k][threadIdx.x + h];
                s[k][threadIdx.x] = (b < s[k][threadIdx.x]) ? b : s[k][threadIdx.x];
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int k = 0; k < 5; k++) part[(long long)k * gridDim.x + blockIdx.x] = s[k][0];
}


// FP32 estimates of cell i's fast-mode candidate a0 and of mc from the float
// inputs ro, tt (certified by `okin`), and whether its momenta are not all
// exactly zero.  When `ok`, both are certified to 1.4e-6: to first order in
// u = 2^-24, mc is within 18u (inputs truncated to 23 bits) or 23u (FP32
// storage: exact momenta and fields, ro and tt within 5u), a0 within 16u.
template <bool MAG, class FA>
__device__ __forceinline__ void cfl_estimate(const FA& U, long long i, float ro, float tt, bool okin, float ddf,
                                             float gam_f, float obeta_f, float& a0, float& mc, bool& ok, bool& nz) {
    const float ru = U.fe(S_RU, i), rv = U.fe(S_RV, i), rw = U.fe(S_RW, i);
    nz = U.nz(S_RU, i) | U.nz(S_RV, i) | U.nz(S_RW, i);  // no short circuit: the loads stay unconditional
    const float ir = __frcp_rn(ro);
    const float sq = __fadd_rn(__fadd_rn(__fmul_rn(ru, ru), __fmul_rn(rv, rv)), __fmul_rn(rw, rw));
    const float uuk = __fmul_rn(__fmul_rn(sq, ir), ir);
    float G = __fmul_rn(gam_f, tt);
    if constexpr (MAG) {
        const float bx = U.fe(S_BX, i), by = U.fe(S_BY, i), bz = U.fe(S_BZ, i);
        const float b2 = __fadd_rn(__fadd_rn(__fmul_rn(bx, bx), __fmul_rn(by, by)), __fmul_rn(bz, bz));
        G = __fadd_rn(G, __fmul_rn(__fmul_rn(obeta_f, b2), ir));
    }
    const float uuf = __fadd_rn(__fadd_rn(uuk, G), __fmul_rn(2.0f, __fsqrt_rn(__fmul_rn(uuk, G))));
    mc = __fdiv_rn(uuk, tt);
    a0 = __fmul_rn(ddf, rsqrtf(uuf));
    ok = okin && (ro >= 0x1p-20f && ro <= 0x1p20f) && (tt >= 0x1p-20f && tt <= 0x1p20f) && isfinite(uuf) &&
         isfinite(mc) && isfinite(a0);
}

// Whether a row takes the filtered path (see k_cfl_rows), with its DD.
__device__ __forceinline__ bool cfl_fast_row(const Grid& g, const Consts& c, int y, int z, double& DDyz) {
    DDyz = cfl_dd_yz(c, y, z);
    const double P1 = 0.5f * DDyz * DDyz * c.REPR * c.CV;  // prefix of cfl_a1
    const double P2 = 0.375f * DDyz * DDyz * c.RE;         // prefix of cfl_a2
    const bool consts_ok = (c.GAMMA >= 0x1p-10 && c.GAMMA <= 0x1p10) && (c.OBETA >= 0.0 && c.OBETA <= 0x1p30);
    return consts_ok && (g.nx <= 3 || !(c.DDXmin < DDyz)) && P1 > 0.0 && P2 > 0.0 && cfl_kappa(c, z) > 0.0;
}

// A row's place, DD and filter test.  A warp works through its rows in batches
// of 32, lane j evaluating the j-th row's FP64 scalars and handing them to the
// others by shuffle: GB300's FP64 pipe retires about 2 lanes per clock per SM,
// so a warp-uniform FP64 expression costs as much as 32 distinct ones.
struct CflRowInfo {
    int y, z;
    double DD;
    bool fast;
};
// row r (of nPy x nPz, y fastest) when r < nrows; otherwise not fast
__device__ __forceinline__ CflRowInfo cfl_row_info(const Grid& g, const Consts& c, long long r, long long nrows) {
    CflRowInfo ri{1, 1, 0.0, false};
    if (r < nrows) {
        const int nPy = g.ny - 2;
        ri.y = 1 + (int)(r % nPy);
        ri.z = 1 + (int)(r / nPy);
        ri.fast = cfl_fast_row(g, c, ri.y, ri.z, ri.DD);
    }
    return ri;
}
__device__ __forceinline__ CflRowInfo cfl_row_from(const CflRowInfo& a, int t) {
    return {__shfl_sync(0xffffffffu, a.y, t), __shfl_sync(0xffffffffu, a.z, t), __shfl_sync(0xffffffffu, a.DD, t),
            __shfl_sync(0xffffffffu, (int)a.fast, t) != 0};
}

// Seeds of the filter: the smallest a0 estimate and the largest mc estimate
// (momenta not all zero) over every kCflSeedStride-th row, as ordered integer
// keys (0 = nothing seen).  Any estimate that some certified cell attains is a
// valid filter base, so the row kernel may start from these.
constexpr int kCflSeedStride = 16;
template <bool MAG, class FA>
__global__ void k_cfl_seed(Grid g, Consts c, FA U, unsigned* seed) {
    const int nPx = g.nx - 2, nPy = g.ny - 2, nPz = g.nz - 2;
    const long long nall = (long long)nPy * nPz;
    const long long nrows = (nall + kCflSeedStride - 1) / kCflSeedStride;
    const int lane = threadIdx.x & 31;
    const long long warps = (long long)gridDim.x * blockDim.x / 32;
    const float gam_f = (float)c.GAMMA, obeta_f = (float)c.OBETA;
    float best_a = INFINITY, best_m = 0.0f;
    for (long long qb = (long long)(blockIdx.x * blockDim.x + threadIdx.x) / 32; qb < nrows; qb += 32 * warps) {
        const long long qj = qb + lane * warps;
        const CflRowInfo mine = cfl_row_info(g, c, qj < nrows ? qj * kCflSeedStride : nall, nall);
        for (int t = 0; t < 32 && qb + t * warps < nrows; t++) {
            const CflRowInfo ri = cfl_row_from(mine, t);
            if (!ri.fast) continue;
            const int y = ri.y, z = ri.z;
            const float ddf = narrow_f64(ri.DD);
            const long long row = (long long)z * g.sz + (long long)y * g.sy;
            const typename FA::Row rk = U.row(z);
#pragma unroll 4
            for (int x = 1 + lane; x <= nPx; x += 32) {  // unrolled: the cells' loads overlap
                float ro, tt, a0, mc;
                bool okin, ok, nz;
                typename FA::Min m;
                U.est_in(rk, row + x, ro, tt, okin, m);
                cfl_estimate<MAG>(U, row + x, ro, tt, okin, ddf, gam_f, obeta_f, a0, mc, ok, nz);
                if (ok) {
                    best_a = fminf(best_a, a0);
                    if (nz) best_m = fmaxf(best_m, mc);
                }
            }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        best_a = fminf(best_a, __shfl_xor_sync(0xffffffffu, best_a, o));
        best_m = fmaxf(best_m, __shfl_xor_sync(0xffffffffu, best_m, o));
    }
    if (lane == 0) {
        // positive floats order like their bit patterns
        if (best_a < INFINITY) atomicMax(&seed[0], 0x7f800000u - __float_as_uint(best_a));
        if (best_m > 0.0f) atomicMax(&seed[1], __float_as_uint(best_m));
    }
}

constexpr int kCflK = 8;                         // cells per lane in one pass over a row
constexpr int kCflWarps = 8;                     // 256 threads
constexpr float kCflTau = 1.52587890625e-05f;    // 2^-16: filter margin, > 2x the approximation error

// The CFL reduction, one warp per (y, z) row of cells.
//
// On a row whose DD is the same in every cell (DDX never below
// min(DDZ[z], DDY[y]); always so on uniform x/y grids) the candidates need no
// per-cell FP64 arithmetic except where they can decide the result:
//   * a1, a2 are products/quotients of ro with positive row constants and a3
//     depends on DD alone; rounding is monotone, so their row minima are the
//     candidates of the row's smallest ro (an exact min: of ro in FP64, of the
//     stored deviation with FP32 storage);
//   * mc and a0 = DD/sqrt(UU') are estimated in FP32 from inputs truncated to
//     23 bits, or from the stored floats with ro and T summed in FP32 with
//     FP32 storage (error below 1.4e-6 for inputs in the accepted ranges); a cell is
//     evaluated exactly when its estimate lies within 2^-16 of the best
//     estimate the warp has seen so far (the running maximum of mc, minimum of
//     a0, the current pass included), or when its estimate is not certified
//     (out-of-range input, non-finite value).  The best estimate seen so far
//     is never better than the best over all of the warp's cells, and the cell
//     holding the warp's exact extremum has an estimate within the error
//     bound of that, so it is always evaluated exactly.
// The exact maximum of mc and minimum of a0 are therefore among the cells
// evaluated exactly, and the result equals the cell-by-cell reduction bit for
// bit; after the first passes only new near-extremes are evaluated.  Rows with varying DD, and launches whose constants break the
// monotonicity (non-positive factors), evaluate every cell exactly.
template <bool MAG, class FA>
__global__ void __launch_bounds__(kCflWarps * 32, 3) k_cfl_rows(Grid g, Consts c, FA U, const unsigned* seed,
                                                             double* part) {
    __shared__ int list[kCflWarps][32 * kCflK];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int nPx = g.nx - 2, nPy = g.ny - 2, nPz = g.nz - 2;
    const long long nrows = (long long)nPy * nPz;
    const double OGAMMA = 1.0f / c.GAMMA;
    const float gam_f = (float)c.GAMMA, obeta_f = (float)c.OBETA;
    double um = 0.0f, w0 = 1e99, w1 = 1e99, w2 = 1e99, w3 = 1e99;
    // the best estimates so far (warp-uniform), starting from the seeds
    float run_a = seed[0] ? __uint_as_float(0x7f800000u - seed[0]) : INFINITY;
    float run_m = seed[1] ? __uint_as_float(seed[1]) : -INFINITY;
    const long long stride = (long long)gridDim.x * kCflWarps;
    for (long long rb = (long long)blockIdx.x * kCflWarps + wid; rb < nrows; rb += 32 * stride) {
        // lane j holds the j-th row of this batch of 32 and, once that row is
        // reduced, its smallest density (stored deviation with FP32 storage)
        const CflRowInfo mine = cfl_row_info(g, c, rb + lane * stride, nrows);
        typename FA::Min mine_ro = INFINITY;
        for (int t = 0; t < 32 && rb + t * stride < nrows; t++) {
            const CflRowInfo ri = cfl_row_from(mine, t);
            const int y = ri.y, z = ri.z;
            const long long row = (long long)z * g.sz + (long long)y * g.sy;
            if (!ri.fast) {
                for (int x = 1 + lane; x <= nPx; x += 32) cfl_cell<MAG>(g, c, U, x, y, z, OGAMMA, um, w0, w1, w2, w3);
                continue;
            }
            const double DDyz = ri.DD;
            typename FA::Min mro = INFINITY;  // no cell yet
            const float ddf = narrow_f64(DDyz);
            const typename FA::Row rk = U.row(z);
            for (int x0 = 1; x0 <= nPx; x0 += 32 * kCflK) {
                float aA[kCflK], mA[kCflK];
                unsigned okm = 0u, nzm = 0u, valid = 0u;
                float Ma = INFINITY, Mm = -INFINITY;
#pragma unroll
                for (int k = 0; k < kCflK; k++) {
                    const int x = x0 + k * 32 + lane;
                    aA[k] = 0.0f;
                    mA[k] = 0.0f;
                    if (x > nPx) continue;
                    valid |= 1u << k;
                    const long long i = row + x;
                    float ro, tt, a0, mc;
                    bool okin, ok, nz;
                    typename FA::Min m;
                    U.est_in(rk, i, ro, tt, okin, m);
                    mro = (m < mro) ? m : mro;
                    cfl_estimate<MAG>(U, i, ro, tt, okin, ddf, gam_f, obeta_f, a0, mc, ok, nz);
                    aA[k] = a0;
                    mA[k] = mc;
                    if (ok) {
                        okm |= 1u << k;
                        Ma = fminf(Ma, a0);
                        if (nz) Mm = fmaxf(Mm, mc);
                    }
                    if (nz) nzm |= 1u << k;
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    Ma = fminf(Ma, __shfl_xor_sync(0xffffffffu, Ma, o));
                    Mm = fmaxf(Mm, __shfl_xor_sync(0xffffffffu, Mm, o));
                }
                run_a = fminf(run_a, Ma);
                run_m = fmaxf(run_m, Mm);
                const float ta = run_a + kCflTau * run_a;
                const float tm = (run_m >= 0x1p-40f) ? run_m - kCflTau * run_m : -INFINITY;
                unsigned cm = 0u;  // this lane's cells to evaluate exactly, bit k
#pragma unroll
                for (int k = 0; k < kCflK; k++) {
                    const bool v = (valid >> k) & 1u, ok = (okm >> k) & 1u, nz = (nzm >> k) & 1u;
                    if (v && (!ok || aA[k] <= ta || (nz && mA[k] >= tm))) cm |= 1u << k;
                }
                // Most passes have no such cell; the compaction (ballots and
                // population counts, the latter on GB300's FP64 pipe) runs
                // only when one has.
                if (__any_sync(0xffffffffu, cm != 0u)) {
                    int n = 0;
#pragma unroll
                    for (int k = 0; k < kCflK; k++) {
                        const bool cand = (cm >> k) & 1u;
                        const unsigned bal = __ballot_sync(0xffffffffu, cand);
                        if (cand) list[wid][n + __popc(bal & ((1u << lane) - 1u))] = x0 + k * 32 + lane;
                        n += __popc(bal);
                    }
                    __syncwarp();
                    for (int j = lane; j < n; j += 32) {
                        const int x = list[wid][j];
                        double mc, UU;
                        cfl_speeds<MAG>(c, U, row + x, z, OGAMMA, mc, UU);
                        um = (um < mc) ? mc : um;
                        const double a0 = DDyz / sqrt(UU);
                        w0 = (a0 < w0) ? a0 : w0;
                    }
                    __syncwarp();
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const typename FA::Min q = __shfl_xor_sync(0xffffffffu, mro, o);
                mro = (q < mro) ? q : mro;
            }
            if (lane == t) mine_ro = mro;
        }
        // the a1..a3 candidates of every fast row of the batch, one row per lane
        if (mine.fast) {
            const double rmin = U.ro_min(mine_ro, mine.z);
            const double a1 = cfl_a1(c, mine.DD, rmin, mine.z), a2 = cfl_a2(c, mine.DD, rmin);
            w1 = (a1 < w1) ? a1 : w1;
            w2 = (a2 < w2) ? a2 : w2;
            if constexpr (MAG) {
                const double a3 = cfl_a3(c, mine.DD);
                w3 = (a3 < w3) ? a3 : w3;
            }
        }
    }
    write_cfl_partials(um, w0, w1, w2, w3, part);
}

// Launch the row reduction with one wave of resident blocks (each warp then
// sees many rows, so its running estimates filter most cells); returns the
// number of partial blocks.
template <class FA>
int launch_cfl_rows_t(bool mag, const Grid& g, const Consts& c, FA U, double* partials, int max_blocks,
                    cudaStream_t st) {
    static int wave[2] = {0, 0};  // per accessor type
    int& w = wave[mag ? 1 : 0];
    if (!w) {
        int dev = 0, sms = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (mag) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cfl_rows<true, FA>, kCflWarps * 32, 0);
        else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cfl_rows<false, FA>, kCflWarps * 32, 0);
        w = (sms > 0 ? sms : 1) * (per_sm > 0 ? per_sm : 1);
    }
    const long long nrows = (long long)(g.ny - 2) * (g.nz - 2);
    long long nb = (nrows + kCflWarps - 1) / kCflWarps;
    if (nb < 1) nb = 1;
    if (nb > w) nb = w;
    if (nb > max_blocks) nb = max_blocks;
    // two seed words after the largest partial block (5 x max_blocks doubles)
    unsigned* seed = reinterpret_cast<unsigned*>(partials + 5 * (size_t)max_blocks);
    cudaMemsetAsync(seed, 0, 2 * sizeof(unsigned), st);
    const long long srows = (nrows + kCflSeedStride - 1) / kCflSeedStride;
    long long sb = (srows * 32 + 255) / 256;
    if (sb > w) sb = w;
    if (sb < 1) sb = 1;
    if (mag) {
        k_cfl_seed<true, FA><<<(int)sb, 256, 0, st>>>(g, c, U, seed);
        k_cfl_rows<true, FA><<<(int)nb, kCflWarps * 32, 0, st>>>(g, c, U, seed, partials);
    } else {
        k_cfl_seed<false, FA><<<(int)sb, 256, 0, st>>>(g, c, U, seed);
        k_cfl_rows<false, FA><<<(int)nb, kCflWarps * 32, 0, st>>>(g, c, U, seed, partials);
    }
    return (int)nb;
}
int launch_cfl_rows(bool mag, const Grid& g, const Consts& c, Fields8 U, double* partials, int max_blocks,
                    cudaStream_t st) {
    return launch_cfl_rows_t(mag, g, c, CflFields64{U}, partials, max_blocks, st);
}

// Reduce the per-block CFL partials (5 x nb) into v[0] = max UMACH^2
// candidate, v[1..4] = min time-step candidates, in thread 0.
__device__ void reduce_cfl_partials(const double* part, int nb, double v[5]) {
    __shared__ double s[5][256];
    v[0] = 0.0;
    for (int k = 1; k < 5; k++) v[k] = 1e99;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) {
        const double a = part[b];
        v[0] = (v[0] < a) ? a : v[0];
        for (int k = 1; k < 5; k++) {
            const double q = part[(long long)k * nb + b];
            v[k] = (q < v[k]) ? q : v[k];
        }
    }
    for (int k = 0; k < 5; k++) s[k][threadIdx.x] = v[k];
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h) {
            const double a = s[0][threadIdx.x + h];
            s[0][threadIdx.x] = (s[0][threadIdx.x] < a) ? a : s[0][threadIdx.x];
            for (int k = 1; k < 5; k++) {
                const double b = s[k][threadIdx.x + h];
                s[k][threadIdx.x] = (b < s[k][threadIdx.x]) ? b : s[k][threadIdx.x];
            }
        }
        __syncthreads();
    }
    for (int k = 0; k < 5; k++) v[k] = s[k][0];
}

__global__ void k_cfl_finish(const double* part, int nb, double* out) {
    double v[5];
    reduce_cfl_partials(part, nb, v);
    if (threadIdx.x == 0)
        for (int k = 0; k < 5; k++) out[k] = v[k];
}

// DT = SFF * min(candidates) as step() forms it (3dmhdsub.h:44,102-104), kept
// in the device record; a DT below 1e-8 (or not a number) halts the run as
// 3dmhd.cpp:292 does: the flag stays set, the record's DT becomes 0 and the
// substage kernels then leave the state unchanged.  TIMC and TIMT advance as
// 3dmhdsub.h:150-152 does once per completed step.
__global__ void k_cfl_record(const double* part, int nb, double sff, int mag, double* rec) {
    double v[5];
    reduce_cfl_partials(part, nb, v);
    if (threadIdx.x != 0) return;
    auto mn = [](double a, double b) { return (b < a) ? b : a; };
    const double dt = mag ? sff * mn(mn(v[1], v[2]), mn(v[3], v[4])) : sff * mn(mn(v[1], v[2]), v[3]);
    const bool stop = rec[3] != 0.0 || !(dt >= 1.0e-8f);
    if (rec[3] == 0.0) {
        rec[4] = dt;
        rec[2] = sqrt(v[0]);
    }
    rec[3] = stop ? 1.0 : 0.0;
    rec[0] = stop ? 0.0 : dt;
    if (!stop) {
        rec[7] += dt;
        rec[1] = rec[6] + rec[7];
        rec[5] += 1.0;
    }
}

int grid_for(long long n, int threads, int cap) {
    long long b = (n + threads - 1) / threads;
    if (b < 1) b = 1;
    if (b > cap) b = cap;
    return (int)b;
}

template <class SW>
void launch_flux(const Grid& g, const Consts& c, Fields8 U, Fields8 F, double* P, double* UU, double* VV, double* WW,
                 cudaStream_t st) {
    const long long ncell = (long long)(g.nx - 2) * (g.ny - 2) * (g.nz - 2);
    k_flux<SW><<<grid_for(ncell, 128, 152 * 64), 128, 0, st>>>(g, c, U, F, P, UU, VV, WW);
}

template <class SW>
void launch_bcon(const Grid& g, const Consts& c, Fields8 U, double timt, cudaStream_t st) {
    const int n = (g.nx - 2) * (g.ny - 2);
    k_bcon<SW><<<(n + 127) / 128, 128, 0, st>>>(g, c, U, timt);
}

}  // namespace

int parity_fluxes(unsigned sw, const Grid& g, const Consts& c, Fields8 U, Fields8 F, double* P, double* UU,
                  double* VV, double* WW, cudaStream_t st) {
    const long long n = (long long)g.nx * g.ny * g.nz;
    k_prep<<<grid_for(n, 256, 152 * 32), 256, 0, st>>>(g, c, U, F.p[F_FW], P, UU, VV, WW);
    MHD_DISPATCH_SW(sw, launch_flux, g, c, U, F, P, UU, VV, WW, st);
    return (int)cudaGetLastError();
}

int parity_fluxes_ext(unsigned sw, const Grid& g, const Consts& c, Fields8 U, Fields8 F, double* RI, double* P,
                      double* UU, double* VV, double* WW, cudaStream_t st) {
    const long long n = (long long)g.nx * g.ny * g.nz;
    k_prep_ext<<<grid_for(n, 256, 152 * 32), 256, 0, st>>>(g, c, U, RI, F.p[F_FW], P, UU, VV, WW);
    Fields8 V = U;
    V.p[S_RO] = RI;  // k_flux reads 1/rho through the RO slot
    MHD_DISPATCH_SW(sw, launch_flux, g, c, V, F, P, UU, VV, WW, st);
    return (int)cudaGetLastError();
}

int parity_rk(int kind, int nf, const Grid& g, Fields8 U, Fields8 Z, Fields8 F, double coef, cudaStream_t st) {
    const long long ncell = (long long)(g.nx - 2) * (g.ny - 2) * (g.nz - 2);
    k_rk<<<grid_for(ncell, 256, 152 * 32), 256, 0, st>>>(kind, nf, g, U, Z, F, coef);
    return (int)cudaGetLastError();
}

int parity_bcon(unsigned sw, const Grid& g, const Consts& c, Fields8 U, double timt, cudaStream_t st) {
    MHD_DISPATCH_SW(sw, launch_bcon, g, c, U, timt, st);
    return (int)cudaGetLastError();
}

int parity_communicate(int nf, const Grid& g, Fields8 U, cudaStream_t st) {
    const long long n = (2LL * g.nx + 2LL * (g.ny - 2)) * g.nz;
    k_comm<<<grid_for(n, 256, 152 * 16), 256, 0, st>>>(nf, g, U);
    return (int)cudaGetLastError();
}

// horizontal_mean (3dmhdsub.h:698-718) of T on every z plane, one thread per
// plane summing in the reference's order (y, then x)
__global__ void k_lrem_ttm_exact(Grid g, const double* TT, double* ttm) {
    const int z = blockIdx.x * blockDim.x + threadIdx.x;
    if (z >= g.nz) return;
    double w = 0;
    for (int y = 1; y < g.ny - 1; y++)
        for (int x = 1; x < g.nx - 1; x++) w += TT[(long long)z * g.sz + (long long)y * g.sy + x];
    ttm[z] = w / (float)((g.nx - 2) * (g.ny - 2));
}

// the same by a block reduction per plane (any summation order)
__global__ void k_lrem_ttm_fast(Grid g, const double* TT, double* ttm) {
    __shared__ double s[256];
    const int z = blockIdx.x;
    const int n = (g.nx - 2) * (g.ny - 2);
    double w = 0;
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const int y = 1 + k / (g.nx - 2), x = 1 + k % (g.nx - 2);
        w += TT[(long long)z * g.sz + (long long)y * g.sy + x];
    }
    s[threadIdx.x] = w;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h) s[threadIdx.x] += s[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) ttm[z] = s[0] / (float)n;
}

// HRAD (3dmhdsub.h:309-312) and G = HRAD - d2(TTM)/dz2 for interior z
__global__ void k_lrem_hrad(Grid g, Consts c, const double* TTM, double* hrad, double* G) {
    const int z = blockIdx.x * blockDim.x + threadIdx.x;
    if (z >= g.nz) return;
    if (z < 1 || z > g.nz - 2) {
        hrad[z] = 0.0;
        G[z] = 0.0;
        return;
    }
    double h = (((TTM[z + 1] - 2.0f * TTM[z] + TTM[z - 1])) * c.h2z * c.dzzdz[z] * c.dzzdz[z] +
                (TTM[z + 1] - TTM[z - 1]) * c.hz * c.d2zzdz2[z]) * c.RKAPA[z];
    h += (TTM[z + 1] - TTM[z - 1]) * c.hz * c.dzzdz[z] * c.DKAPA[z];
    hrad[z] = h;
    const double dz = c.dzzdz[z];
    const double d2m = ((TTM[z + 1] - TTM[z - 1]) * c.d2zzdz2[z]) * c.hz +
                       (((TTM[z + 1] - 2 * TTM[z]) + TTM[z - 1]) * (dz * dz)) * c.h2z;
    G[z] = h - d2m;
}

int parity_cfl(bool mag, const Grid& g, const Consts& c, Fields8 U, double* partials, int max_blocks, double* out5,
               cudaStream_t st) {
    const int nb = launch_cfl_rows(mag, g, c, U, partials, max_blocks, st);
    k_cfl_finish<<<1, 256, 0, st>>>(partials, nb, out5);
    return (int)cudaGetLastError();
}

int cfl_dt_on_device(bool mag, const Grid& g, const Consts& c, Fields8 U, double* partials, int max_blocks,
                     double* rec, cudaStream_t st) {
    const int nb = launch_cfl_rows(mag, g, c, U, partials, max_blocks, st);
    k_cfl_record<<<1, 256, 0, st>>>(partials, nb, c.SFF, mag ? 1 : 0, rec);
    return (int)cudaGetLastError();
}

int lrem_hrad_from_means(const Grid& g, const Consts& c, double* buf, cudaStream_t st) {
    k_lrem_hrad<<<(g.nz + 63) / 64, 64, 0, st>>>(g, c, buf, buf + g.nz, buf + 2 * g.nz);
    return (int)cudaGetLastError();
}

int lrem_profiles(const Grid& g, const Consts& c, const double* TT, double* buf, bool exact, cudaStream_t st) {
    double *ttm = buf, *hrad = buf + g.nz, *G = buf + 2 * g.nz;
    if (exact) k_lrem_ttm_exact<<<(g.nz + 63) / 64, 64, 0, st>>>(g, TT, ttm);
    else k_lrem_ttm_fast<<<g.nz, 256, 0, st>>>(g, TT, ttm);
    k_lrem_hrad<<<(g.nz + 63) / 64, 64, 0, st>>>(g, c, ttm, hrad, G);
    return (int)cudaGetLastError();
}

int cfl32_rows(bool mag, const Grid& g, const Consts& c, Fields8f U, const double* bgR, const double* bgT,
               double* partials, int max_blocks, double* out5, cudaStream_t st) {
    const int nb = launch_cfl_rows_t(mag, g, c, CflFields32{U, bgR, bgT}, partials, max_blocks, st);
    k_cfl_finish<<<1, 256, 0, st>>>(partials, nb, out5);
    return (int)cudaGetLastError();
}

int cfl32_dt_on_device(bool mag, const Grid& g, const Consts& c, Fields8f U, const double* bgR, const double* bgT,
                       double* partials, int max_blocks, double* rec, cudaStream_t st) {
    const int nb = launch_cfl_rows_t(mag, g, c, CflFields32{U, bgR, bgT}, partials, max_blocks, st);
    k_cfl_record<<<1, 256, 0, st>>>(partials, nb, c.SFF, mag ? 1 : 0, rec);
    return (int)cudaGetLastError();
}

}  // namespace mhd
