// mhd_static.cu -- the reference's fresh-start initial state, Static()
// (3dmhdphsic.h:549-763) followed by communicate(), computed on the host for a
// caller that starts runs without the reference's driver.  No device work.
//
// Static() builds the hydrostatic background (with lRem: the ODE background
// of getbackground below, which also gives the conductivity profile and the
// wall values, mhd_static_lrem_profile) by integrating
//   dY0/dzz = THETA / kappa(zz) / dzzdz,  dY1/dzz = GRAV / (1 + Y0) / dzzdz
// (derivs, 3dmhdphsic.h:347-355) over the computational coordinate, one
// Bulirsch-Stoer step per grid interval (bsstep / mmid / rzextr,
// 3dmhdphsic.h:230-344: modified midpoint plus rational extrapolation),
// T = 1 + Y0, rho = exp(Y1) / (1 + Y0); with lShr the background is T = rho = 1.
// With lMag and AMPB != 0 a Gaussian Bx layer is added and rho lowered to keep
// the total pressure; with AMPB = 0 (and no flux tubes) the field is zero.
// With AMPT != 0 the temperature (lShr: RV) takes multiplicative noise from
// the reference's RAN2 generator (3dmhdphsic.h:523-547), drawn by rank 0 z rank
// by z rank, local plane, y rank, row, column; ranks own consecutive planes
// and rows, so that is global plane, row, column order on every rank grid.
// The Bx layer does depend on the z split: every rank fills its local planes
// 2 .. nRz+1 (3dmhdphsic.h:685-700), so the first interior plane of every z
// rank but the lowest keeps no layer, and the top ghost plane has one.
// The expressions keep the reference's float literals and evaluation order so
// that the state equals the reference's bit for bit.
#include "mhd_context.h"

#include <algorithm>
#include <cmath>
#include <vector>

namespace {

struct StaticModel {
    double THETA, GRAV, zMax, PZP, SIGMA, RKAPST;
};

// dY/dz of the background at computational coordinate zz (derivs with the
// uniform grid mapping z = zz zMax of mkGrid, nGrid = 0; kappa from PZP, SIGMA)
void background_slope(const StaticModel& m, double zz, const double* Y, double* D) {
    const double dzzdz = 1.0f / m.zMax;
    double rkap = 1.0f;
    if (m.PZP != 0.0) rkap += (m.RKAPST - 1.0f) / 2.0f * (1.0f + std::tanh((zz - m.PZP) / m.SIGMA));
    D[0] = m.THETA / rkap / dzzdz;
    D[1] = m.GRAV / (1.0f + Y[0]) / dzzdz;
}

// modified midpoint over [xs, xs + htot] in nstp substeps
void midpoint(const StaticModel& m, const double* y, const double* dydx, double xs, double htot, int nstp,
              double* yout) {
    const double h = htot / nstp;
    double x = xs + h;
    double ym[2], yn[2];
    for (int i = 0; i < 2; i++) {
        ym[i] = y[i];
        yn[i] = y[i] + h * dydx[i];
    }
    background_slope(m, x, yn, yout);
    const double h2 = 2.0f * h;
    for (int n = 2; n <= nstp; n++) {
        for (int i = 0; i < 2; i++) {
            const double swap = ym[i] + h2 * yout[i];
            ym[i] = yn[i];
            yn[i] = swap;
        }
        x = x + h;
        background_slope(m, x, yn, yout);
    }
    for (int i = 0; i < 2; i++) yout[i] = 0.5f * (ym[i] + yn[i] + h * yout[i]);
}

// Rational extrapolation of the midpoint results to zero step size.
struct Extrapolator {
    static constexpr int kUse = 7;
    double xs[11] = {}, fx[kUse] = {};
    double d[2][kUse] = {};
    void add(int iest, double xest, const double* yest, double* yz, double* dy) {
        xs[iest] = xest;
        if (iest == 0) {
            for (int j = 0; j < 2; j++) yz[j] = d[j][0] = dy[j] = yest[j];
            return;
        }
        const int m1 = std::min(iest + 1, kUse);
        for (int k = 1; k < m1; k++) fx[k] = xs[iest - k] / xest;
        for (int j = 0; j < 2; j++) {
            double yy = yest[j], v = d[j][0], c = yy, ddy = 0.0;
            d[j][0] = yy;
            for (int k = 1; k < m1; k++) {
                const double b1 = fx[k] * v;
                double b = b1 - c;
                if (b != 0.0) {
                    b = (c - v) / b;
                    ddy = c * b;
                    c = b1 * b;
                } else {
                    ddy = v;
                }
                v = d[j][k];
                d[j][k] = ddy;
                yy = yy + ddy;
            }
            dy[j] = ddy;
            yz[j] = yy;
        }
    }
};

// One Bulirsch-Stoer step of size htry from x; returns the step taken.
double bs_step(const StaticModel& m, double* y, const double* dydx, double& x, double htry, double eps) {
    static const int nseq[11] = {2, 4, 6, 8, 12, 16, 24, 32, 48, 64, 96};
    double h = htry;
    const double xsav = x;
    const double ysav[2] = {y[0], y[1]}, dysav[2] = {dydx[0], dydx[1]};
    for (;;) {
        Extrapolator ex;
        for (int i = 0; i < 11; i++) {
            double yseq[2], yerr[2];
            midpoint(m, ysav, dysav, xsav, h, nseq[i], yseq);
            const double q = h / nseq[i];
            ex.add(i, q * q, yseq, y, yerr);
            double errmax = 0.0f;
            for (int j = 0; j < 2; j++) errmax = std::max(errmax, std::abs(yerr[j] / y[j]));
            errmax /= eps;
            if (errmax < 1) {
                x = x + h;
                return h;
            }
        }
        h = 0.25f * h / std::pow(2.0f, (11 - 7) / 2);
        if (x + h == x) return 0.0;
    }
}

// ---- lRem: the background of getbackground (3dmhdphsic.h:357-362) --------
// An ODE in the physical depth x for (T, P): dT/dx = min(0.4 / kappa, 0.41)
// (radiative gradient capped at the adiabatic one), dP/dx = P / T, with the
// conductivity kappa = rho + (1.25 - rho) exp(-5 x) (kappa and derivs1,
// 3dmhdphsic.h:389-405), integrated from x = 2 (T = P = 1) to each level by
// classical RK4 steps under step doubling with error control (RK4, RKQC and
// ODEINT, 3dmhdphsic.h:409-522, the published Numerical Recipes scheme).
double lrem_kappa(double z, double rho) { return rho + (1.25f - rho) * std::exp(-5.0f * z); }

void lrem_slope(double x, const double* y, double* d) {
    const double nad = 0.41f, os = 1.0f;
    const double nrad = 0.4f / lrem_kappa(x, y[1] / y[0]);
    d[0] = (nrad <= os * nad) ? nrad : nad;
    d[1] = y[1] / y[0];
}

void lrem_rk4(const double* y, const double* dydx, double x, double h, double* yout) {
    double yt[2], dyt[2], dym[2];
    const double hh = h * 0.5f, h6 = h / 6.0f, xh = x + hh;
    for (int i = 0; i < 2; i++) yt[i] = y[i] + hh * dydx[i];
    lrem_slope(xh, yt, dyt);
    for (int i = 0; i < 2; i++) yt[i] = y[i] + hh * dyt[i];
    lrem_slope(xh, yt, dym);
    for (int i = 0; i < 2; i++) {
        yt[i] = y[i] + h * dym[i];
        dym[i] = dyt[i] + dym[i];
    }
    lrem_slope(x + h, yt, dyt);
    for (int i = 0; i < 2; i++) yout[i] = y[i] + h6 * (dydx[i] + dyt[i] + 2.0f * dym[i]);
}

// One controlled step (two half steps against one full step); false where
// the reference aborts ("Stepsize not significant in RKQC").
bool lrem_controlled_step(double* y, double* dydx, double& x, double htry, double eps, const double* yscal,
                          double& hdid, double& hnext) {
    const double fcor = 1.0f / 15.0f, safety = 0.9f, errcon = 6.0e-4f, pgrow = -0.20f, pshrnk = -0.25f;
    const double xsav = x;
    const double ysav[2] = {y[0], y[1]}, dysav[2] = {dydx[0], dydx[1]};
    double ytemp[2];
    double h = htry;
    for (;;) {
        const double hh = 0.5f * h;
        lrem_rk4(ysav, dysav, xsav, hh, ytemp);
        x = xsav + hh;
        lrem_slope(x, ytemp, dydx);
        lrem_rk4(ytemp, dydx, x, hh, y);
        x = xsav + h;
        if (x == xsav) return false;
        lrem_rk4(ysav, dysav, xsav, h, ytemp);
        double errmax = 0.0f;
        for (int i = 0; i < 2; i++) {
            ytemp[i] = y[i] - ytemp[i];
            errmax = std::max(errmax, std::fabs(ytemp[i] / yscal[i]));
        }
        errmax = errmax / eps;
        if (errmax > 1.0) {
            h = safety * h * std::pow(errmax, pshrnk);
        } else {
            hdid = h;
            hnext = errmax > errcon ? safety * h * std::pow(errmax, pgrow) : 4.0f * h;
            break;
        }
    }
    for (int i = 0; i < 2; i++) y[i] += ytemp[i] * fcor;
    return true;
}

// T and rho at depth x; false where the reference aborts.
bool lrem_background(double x, double& t, double& rho) {
    const double tiny = 1.0e-30f, h1 = 1e-4, hmin = 1e-50, eps = 1e-8;
    const double x1 = 2.0f, x2 = x;
    double y[2] = {1.0, 1.0}, dydx[2], yscal[2];
    double xc = x1, h = (x2 > x1) ? h1 : -h1;
    for (int nstp = 1; nstp <= 1000; nstp++) {
        lrem_slope(xc, y, dydx);
        for (int i = 0; i < 2; i++) yscal[i] = std::abs(y[i]) + std::abs(h * dydx[i]) + tiny;
        if ((xc + h - x2) * (xc + h - x1) > 0) h = x2 - xc;
        double hdid, hnext;
        if (!lrem_controlled_step(y, dydx, xc, h, eps, yscal, hdid, hnext)) return false;
        if ((xc - x2) * (x2 - x1) >= 0) {
            t = y[0];
            rho = y[1] / y[0];
            return true;
        }
        if (std::abs(hnext) < hmin) return false;
        h = hnext;
    }
    return false;  // "Too many steps."
}

// The lRem part of Static() (3dmhdphsic.h:565-594): T, rho and the scaled
// conductivity RK with its z derivative DRK on the nPz levels, and the wall
// values TU, DZTU, DZTB.  False where the reference aborts.
bool lrem_profile(const mhd_params* p, double zMax, std::vector<double>& T, std::vector<double>& R,
                  std::vector<double>& RK, std::vector<double>& DRK, double walls[3]) {
    const int nPz = p->nPz;
    mhd_constants k;
    mhd_compute_constants(p, &k);
    T.assign(nPz, 0.0);
    R.assign(nPz, 0.0);
    RK.assign(nPz, 0.0);
    DRK.assign(nPz, 0.0);
    for (int j = 0; j < nPz; j++) {
        const double code = static_cast<float>(j) / static_cast<float>(nPz - 1);
        const double sz = code * zMax;  // mkGrid with a uniform grid
        if (!lrem_background(sz, T[j], R[j])) return false;
        RK[j] = lrem_kappa(sz, R[j]);
        RK[j] *= 8.07f * p->THETA * k.REPR;
    }
    const double sdzzdz = 1.0f / zMax;
    DRK[0] = (-3.0f * RK[0] + 4.0f * RK[1] - RK[2]) * k.hz * sdzzdz;
    for (int j = 1; j < nPz - 1; j++) DRK[j] = (RK[j + 1] - RK[j - 1]) * k.hz * sdzzdz;
    DRK[nPz - 1] = (3.0f * RK[nPz - 1] - 4.0f * RK[nPz - 2] + RK[nPz - 3]) * k.hz * sdzzdz;
    walls[0] = T[0];
    walls[1] = T[0] - 4.0f / 3.0f * T[1] + 1.0f / 3.0f * T[2];
    walls[2] = T[nPz - 1] - 4.0f / 3.0f * T[nPz - 2] + 1.0f / 3.0f * T[nPz - 3];
    return true;
}

// RAN2 (3dmhdphsic.h:523-547): a shuffled linear congruential generator
struct Ran2 {
    static constexpr int M = 714025, IA = 1366, IC = 150889;
    int iiy = 0, iir[97] = {};
    int idum;
    explicit Ran2(int seed) : idum(seed) {}
    double next() {
        if (idum < 0) {
            idum = (int)std::fmod(IC - idum, M);
            for (int j = 0; j < 97; j++) {
                idum = (int)std::fmod(IA * idum + IC, M);
                iir[j] = idum;
            }
            idum = (int)std::fmod(IA * idum + IC, M);
            iiy = idum;
        }
        const int j = (97 * iiy) / M;
        iiy = iir[j];
        const double rm = 1.0f / M;
        const double v = float(iiy) * rm;
        idum = (IA * idum + IC) % M;
        iir[j] = idum;
        return v;
    }
};

}  // namespace

extern "C" int mhd_static_state(const mhd_params* p, const mhd_static_params* s, double* state) {
    if (!p || !s || !state || !s->ZEE) return MHD_ERR_INVALID;
    const bool rem = (p->switches & MHD_SW_LREM) != 0;
    if (rem && (p->switches & MHD_SW_LSHR)) return MHD_ERR_UNSUPPORTED;
    if (s->nTube < 0 || s->nTube > 5) return MHD_ERR_INVALID;
    // tube models 1-5 leave the reference without a state (abort or no build)
    if (s->nTube != 0 && (p->switches & MHD_SW_LMAG) && s->AMPB == 0.0) return MHD_ERR_UNSUPPORTED;
    const int nPx = p->nPx, nPy = p->nPy, nPz = p->nPz, nPEy = s->nPEy, nPEz = s->nPEz;
    if (nPx < 2 || nPy < 2 || nPz < 4 || nPEy < 1 || nPEz < 1 || nPy % nPEy || nPz % nPEz) return MHD_ERR_INVALID;
    const bool mag = (p->switches & MHD_SW_LMAG) != 0, shr = (p->switches & MHD_SW_LSHR) != 0;
    const int nx = nPx + 2, ny = nPy + 2, nz = nPz + 2, nf = mag ? 8 : 5;
    const size_t ncell = (size_t)nx * ny * nz;
    std::fill(state, state + (size_t)nf * ncell, 0.0);
    auto F = [&](int f, int z, int y, int x) -> double& { return state[(size_t)f * ncell + ((size_t)z * ny + y) * nx + x]; };

    // background profile T[k], R[k] on the nPz interior levels
    std::vector<double> T(nPz, 1.0), R(nPz, 1.0);
    if (rem) {
        std::vector<double> RK, DRK;
        double walls[3];
        if (!lrem_profile(p, s->zMax, T, R, RK, DRK, walls)) return MHD_ERR_NUMERIC;
    } else if (!shr) {
        StaticModel m{p->THETA, p->GRAV, s->zMax, s->PZP, s->SIGMA,
                      p->GRAV == 0.0 ? 1.0f : (s->POLYS + 1.0f) * p->THETA / p->GRAV};
        const double eps = 1.0E-12f, dzz = 1.0f / float(nPz - 1);
        double Y[2] = {0.0f, 0.0f}, D[2], zz = 0.0f;
        for (int k = 1; k < nPz; k++) {
            background_slope(m, zz, Y, D);
            if (bs_step(m, Y, D, zz, dzz, eps) != dzz) return MHD_ERR_NUMERIC;
            T[k] = 1.0f + Y[0];
            R[k] = std::exp(Y[1]) / (1.0f + Y[0]);
        }
    }
    // plane gz of the global domain takes level gz - 1, the wall ghosts repeat
    // the walls (3dmhdphsic.h:616-681 for nPEz >= 2)
    for (int z = 0; z < nz; z++) {
        const int k = std::min(std::max(z - 1, 0), nPz - 1);
        for (int y = 1; y <= nPy; y++)
            for (int x = 1; x <= nPx; x++) {
                F(MHD_TT, z, y, x) = T[k];
                F(MHD_RO, z, y, x) = R[k];
            }
    }
    // Bx layer (3dmhdphsic.h:683-700) on local planes 2 .. nRz+1 of every z rank
    if (mag && s->AMPB != 0.0) {
        const double CLN = -4.0f * std::log(2.0f) / (s->BFH * s->BFH);
        const double obeta = 2.0f / p->BETA;  // OBETA, 3dmhd.cpp:459
        const int nRz = nPz / nPEz;
        for (int z = 2; z <= nPz + 1; z++) {
            if (z <= nPz && (z - 1) % nRz == 0) continue;  // local plane 1 of its z rank
            const double d = s->ZEE[z] - s->BZP;
            const double bx = s->AMPB * std::exp(CLN * (d * d));
            for (int y = 0; y < ny; y++)
                for (int x = 0; x < nx; x++) F(MHD_BX, z, y, x) = bx;
            for (int y = 1; y <= nPy; y++)
                for (int x = 1; x <= nPx; x++)
                    F(MHD_RO, z, y, x) -= (F(MHD_BX, z, y, x) * F(MHD_BX, z, y, x) / F(MHD_TT, z, y, x)) * obeta;
        }
    }
    // noise (3dmhdphsic.h:705-744): rank 0 draws for every z rank, local
    // interior plane and y rank, rows y, columns x
    if (s->AMPT != 0.0) {
        Ran2 rng(-62659);
        const int nRy = nPy / nPEy, nRz = nPz / nPEz;
        for (int nnz = 0; nnz < nPEz; nnz++)
            for (int k = 1; k <= nRz; k++)
                for (int nny = 0; nny < nPEy; nny++)
                    for (int y = 1; y <= nRy; y++)
                        for (int x = 1; x <= nPx; x++) {
                            const double w = 1.0f + s->AMPT * (rng.next() - 0.5E00);
                            const int gz = nnz * nRz + k, gy = nny * nRy + y;
                            if (!shr) F(MHD_TT, gz, gy, x) = F(MHD_TT, gz, gy, x) * w;
                            else F(MHD_RV, gz, gy, x) = F(MHD_RV, gz, gy, x) + w - 1.0f;
                        }
    }
    // x / y ghosts as periodic images (communicate(), 3dmhdmpi.h:11-143); the
    // z planes ranks exchange there are interior planes here
    for (int f = 0; f < nf; f++)
        for (int z = 0; z < nz; z++) {
            for (int x = 0; x < nx; x++) {
                F(f, z, 0, x) = F(f, z, ny - 2, x);
                F(f, z, ny - 1, x) = F(f, z, 1, x);
            }
            for (int y = 0; y < ny; y++) {
                F(f, z, y, 0) = F(f, z, y, nx - 2);
                F(f, z, y, nx - 1) = F(f, z, y, 1);
            }
        }
    return MHD_OK;
}

extern "C" int mhd_static_lrem_profile(const mhd_params* p, const mhd_static_params* s, double* rkapa, double* dkapa,
                                       double* walls) {
    if (!p || !s || !rkapa || !dkapa || !walls) return MHD_ERR_INVALID;
    if (!(p->switches & MHD_SW_LREM) || (p->switches & MHD_SW_LSHR)) return MHD_ERR_INVALID;
    if (p->nPz < 4) return MHD_ERR_INVALID;
    std::vector<double> T, R, RK, DRK;
    if (!lrem_profile(p, s->zMax, T, R, RK, DRK, walls)) return MHD_ERR_NUMERIC;
    // global plane gz takes level gz - 1; the wall ghosts repeat the walls
    // (RKAPA = RK, DKAPA = DRK of Static()'s plane assignment, 3dmhdphsic.h:616-681)
    const int nz = p->nPz + 2;
    for (int z = 0; z < nz; z++) {
        const int j = std::min(std::max(z - 1, 0), p->nPz - 1);
        rkapa[z] = RK[j];
        dkapa[z] = DRK[j];
    }
    return MHD_OK;
}
