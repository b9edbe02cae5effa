/*
 * mhd_oracle.c -- CPU restatement of the reference 3dmhd hot path (the
 * checker; see mhd_oracle.h).  Compile with -O2 -ffp-contract=off (and
 * optionally -fopenmp: every sweep is independent per cell, so threading
 * does not change a bit).
 *
 * Conventions, all from 3dmhdutils.h:
 *   f[z][y][x], x fastest; derivative of F along u at a node:
 *     D1_u F = ((F[u+1] - F[u-1]) * duudu[u]) * hu               (:195-199)
 *     D2_u F = ((F[u+1]-F[u-1]) * d2uudu2[u]) * hu
 *              + (((F[u+1] - 2F) + F[u-1]) * (duudu*duudu)) * h2u  (:215-220)
 *   products associate left to right, the scale factor is applied last and
 *   the result is set, added or subtracted (oper<SET|ADD|SUB>, :126-129).
 *   A scale of 1 is dropped (x*1 == x exactly) and -1 becomes a negation.
 * Ranges (3dmhdutils.h:20-25): R is the interior including the wall planes,
 * EXT adds every ghost, EXT_X / EXT_Y / EXT_XY add the x / y / both ghosts.
 */
#include "mhd_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <stdio.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#define ORC_PRAGMA(x) _Pragma(#x)
#else
#define ORC_PRAGMA(x)
#endif

/* square() of 3dmhdutils.h */
static inline double sq(double v) { return v * v; }

#define SWEEP(...) SWEEP_(__VA_ARGS__)
#define SWEEP_(Z0, Z1, Y0, Y1, X0, X1, ...)                                     \
    do {                                                                        \
        ORC_PRAGMA(omp parallel for schedule(static))                           \
        for (int z = (Z0); z < (Z1); z++)                                       \
            for (int y = (Y0); y < (Y1); y++)                                   \
                for (int x = (X0); x < (X1); x++) {                             \
                    const size_t i = ((size_t)z * (size_t)ny + (size_t)y) * (size_t)nx + (size_t)x; \
                    (void)i;                                                    \
                    __VA_ARGS__;                                                \
                }                                                               \
    } while (0)

#define R_ 1, nz - 1, 1, ny - 1, 1, nx - 1
#define EXT_ 0, nz, 0, ny, 0, nx
#define EXT_X_ 1, nz - 1, 1, ny - 1, 0, nx
#define EXT_Y_ 1, nz - 1, 0, ny, 1, nx - 1
#define EXT_XY_ 1, nz - 1, 0, ny, 0, nx

/* central differences of F at flat index i */
#define DX(F) ((F)[i + 1] - (F)[i - 1])
#define DY(F) ((F)[i + sy] - (F)[i - sy])
#define DZ(F) ((F)[i + sz] - (F)[i - sz])
#define D1X(F) ((DX(F) * p->dxxdx[x]) * p->hx)
#define D1Y(F) ((DY(F) * p->dyydy[y]) * p->hy)
#define D1Z(F) ((DZ(F) * p->dzzdz[z]) * p->hz)
#define D2X(F) ((DX(F) * p->d2xxdx2[x]) * p->hx + ((((F)[i + 1] - 2 * (F)[i]) + (F)[i - 1]) * (p->dxxdx[x] * p->dxxdx[x])) * p->h2x)
#define D2Y(F) ((DY(F) * p->d2yydy2[y]) * p->hy + ((((F)[i + sy] - 2 * (F)[i]) + (F)[i - sy]) * (p->dyydy[y] * p->dyydy[y])) * p->h2y)
#define D2Z(F) ((DZ(F) * p->d2zzdz2[z]) * p->hz + ((((F)[i + sz] - 2 * (F)[i]) + (F)[i - sz]) * (p->dzzdz[z] * p->dzzdz[z])) * p->h2z)
/* derivative of a product, func_mul_d1 (3dmhdutils.h:236-239) */
#define MDX(F, G) ((((F)[i + 1] * (G)[i + 1] - (F)[i - 1] * (G)[i - 1]) * p->dxxdx[x]) * p->hx)
#define MDY(F, G) ((((F)[i + sy] * (G)[i + sy] - (F)[i - sy] * (G)[i - sy]) * p->dyydy[y]) * p->hy)
#define MDZ(F, G) ((((F)[i + sz] * (G)[i + sz] - (F)[i - sz] * (G)[i - sz]) * p->dzzdz[z]) * p->hz)

#define DECL_DIMS                           \
    const int nx = p->nx, ny = p->ny, nz = p->nz; \
    const size_t sy = (size_t)nx;           \
    const size_t sz = (size_t)nx * (size_t)ny; \
    (void)sy;                               \
    (void)sz

static void set_threads(const orc_params* p) {
#ifdef _OPENMP
    if (p->nthreads > 0) omp_set_num_threads(p->nthreads);
#else
    (void)p;
#endif
}

void orc_set_constants(orc_params* p, int nPx, int nPy, int nPz) {
    /* 3dmhd.cpp:354-369: constants evaluated in single precision, then widened */
    p->C13 = 1.0f / 3.0f;
    p->C23 = 2.0f * p->C13;
    p->C43 = 4.0f * p->C13;
    p->GAM1 = 8.0f / 15.0f;
    p->GAM2 = 5.0f / 12.0f;
    p->GAM3 = 3.0f / 4.0f;
    p->ZETA1 = -17.0f / 60.0f;
    p->ZETA2 = -5.0f / 12.0f;
    p->hx = 0.5f * (float)(nPx - 1);
    p->h2x = (float)(nPx - 1) * (float)(nPx - 1);
    p->hy = 0.5f * (float)(nPy - 1);
    p->h2y = (float)(nPy - 1) * (float)(nPy - 1);
    p->hz = 0.5f * (float)(nPz - 1);
    p->h2z = (float)(nPz - 1) * (float)(nPz - 1);
    p->nPz = nPz;
    /* 3dmhd.cpp:432-438,451-459 */
    if (p->lRot) {
        p->OMX = sin(p->ANG) / p->RY;
        p->OMZ = cos(p->ANG) / p->RY;
    } else {
        p->OMX = 0.0f;
        p->OMZ = 0.0f;
    }
    p->REPR = p->RE * p->PR;
    p->ORE = 1.0f / p->RE;
    p->ORM = 1.0f / p->RM;
    p->OBETA = 2.0f / p->BETA;
    /* 3dmhd.cpp:144-145 */
    p->CV = 1.0f / (p->GAMMA - 1.0f);
    p->OCV = 1.0f / p->CV;
}

/* fluxes(): 3dmhdsub.h:194-696 for ixCon=iyCon=0, iD=0, !lRem, RLAX=0, iTCon!=2 */
int orc_fluxes(const orc_params* p, orc_fields* f) {
    DECL_DIMS;
    set_threads(p);
    double *RU = f->a[ORC_RU], *RV = f->a[ORC_RV], *RW = f->a[ORC_RW], *TT = f->a[ORC_TT], *RO = f->a[ORC_RO];
    double *BX = f->a[ORC_BX], *BY = f->a[ORC_BY], *BZ = f->a[ORC_BZ];
    double *FU = f->a[ORC_FU], *FV = f->a[ORC_FV], *FW = f->a[ORC_FW], *FR = f->a[ORC_FR], *FT = f->a[ORC_FT];
    double *WW1 = f->a[ORC_WW1], *WW2 = f->a[ORC_WW2], *WW3 = f->a[ORC_WW3];
    double *UU = f->a[ORC_UU], *VV = f->a[ORC_VV], *WW = f->a[ORC_WW];
    const int zl = 1, zr = nz - 1;
    double tmp;

    /* continuity, 3dmhdsub.h:204-227 */
    SWEEP(R_, FR[i] = -D1X(RU));
    SWEEP(R_, FR[i] -= D1Y(RV));
    SWEEP(R_, WW1[i] = D1Z(RW));
    {
        const double TMPZ = p->hz * p->dzzdz[zl];
        SWEEP(zl, zl + 1, 1, ny - 1, 1, nx - 1, WW1[i] = (4.0f * RW[i + sz] - RW[i + 2 * sz]) * TMPZ);
    }
    {
        const double TMPZ = p->hz * p->dzzdz[zr - 1];
        SWEEP(zr - 1, zr, 1, ny - 1, 1, nx - 1, WW1[i] = (RW[i - 2 * sz] - 4.0f * RW[i - sz]) * TMPZ);
    }
    SWEEP(R_, FR[i] -= WW1[i]);

    /* lRem: the wall ghost planes of RO take the second interior plane,
     * 3dmhdsub.h:229-238 (the horizontal mean computed after it there is
     * only used with iD != 0) */
    if (p->lRem) {
        memcpy(RO, RO + 2 * sz, sizeof(double) * sz);
        memcpy(RO + (size_t)(nz - 1) * sz, RO + (size_t)(nz - 3) * sz, sizeof(double) * sz);
    }

    /* pressure, gravity and 1/rho in place, 3dmhdsub.h:266-272 */
    SWEEP(R_, FW[i] = RO[i] * p->GRAV);
    SWEEP(EXT_, WW1[i] = RO[i] * TT[i]);
    SWEEP(EXT_, RO[i] = 1.0f / RO[i]);
    SWEEP(R_, FW[i] -= D1Z(WW1));
    SWEEP(R_, FV[i] = -D1Y(WW1));
    SWEEP(R_, FU[i] = -D1X(WW1));

    /* velocities, 3dmhdsub.h:274-276 */
    SWEEP(EXT_, UU[i] = RU[i] * RO[i]; VV[i] = RV[i] * RO[i]; WW[i] = RW[i] * RO[i]);

    /* momentum advection, 3dmhdsub.h:279-289 */
    SWEEP(R_, FU[i] -= MDX(RU, UU));
    SWEEP(R_, FU[i] -= MDY(RU, VV));
    SWEEP(R_, FU[i] -= MDZ(RU, WW));
    SWEEP(R_, FV[i] -= MDX(RV, UU));
    SWEEP(R_, FV[i] -= MDY(RV, VV));
    SWEEP(R_, FV[i] -= MDZ(RV, WW));
    SWEEP(R_, FW[i] -= MDX(RW, UU));
    SWEEP(R_, FW[i] -= MDY(RW, VV));
    SWEEP(R_, FW[i] -= MDZ(RW, WW));

    /* temperature advection, 3dmhdsub.h:293-296 */
    double* TTM = NULL;
    if (!p->lShr) {
        SWEEP(R_, FT[i] = -(D1X(TT) * UU[i]));
        SWEEP(R_, FT[i] -= D1Y(TT) * VV[i]);
        SWEEP(R_, FT[i] -= D1Z(TT) * WW[i]);
        if (p->lRem) {
            /* horizontal_mean (3dmhdsub.h:698-718, one y rank) and WW1 = TT - TTM */
            TTM = (double*)calloc((size_t)nz, sizeof(double));
            for (int z = 0; z < nz; z++) {
                double w = 0;
                for (int y = 1; y < ny - 1; y++)
                    for (int x = 1; x < nx - 1; x++) w += TT[((size_t)z * ny + y) * nx + x];
                TTM[z] = w / (float)((nx - 2) * (ny - 2));
            }
            SWEEP(EXT_, WW1[i] = TT[i] - TTM[z]);
        }
    }

    tmp = p->OCV / p->REPR;
    if (p->lRem && TTM) {
        /* conduction of the deviation plus the mean profile's, 3dmhdsub.h:304-313 */
        SWEEP(R_, FT[i] += (D2X(WW1) * RO[i]) * tmp);
        SWEEP(R_, FT[i] += (D2Y(WW1) * RO[i]) * tmp);
        SWEEP(R_, FT[i] += (D2Z(WW1) * RO[i]) * tmp);
        double* HRAD = (double*)calloc((size_t)nz, sizeof(double));
        for (int z = zl; z < zr; z++) {
            HRAD[z] = (((TTM[z + 1] - 2.0f * TTM[z] + TTM[z - 1])) * p->h2z * p->dzzdz[z] * p->dzzdz[z] +
                       (TTM[z + 1] - TTM[z - 1]) * p->hz * p->d2zzdz2[z]) * p->RKAPA[z];
            HRAD[z] += (TTM[z + 1] - TTM[z - 1]) * p->hz * p->dzzdz[z] * p->DKAPA[z];
        }
        SWEEP(R_, FT[i] += (RO[i] * HRAD[z]) * tmp);
        free(HRAD);
    } else {
        /* conduction, 3dmhdsub.h:315-319 */
        SWEEP(R_, FT[i] += ((D2X(TT) * RO[i]) * p->RKAPA[z]) * tmp);
        SWEEP(R_, FT[i] += ((D2Y(TT) * RO[i]) * p->RKAPA[z]) * tmp);
        SWEEP(R_, FT[i] += ((D2Z(TT) * RO[i]) * p->RKAPA[z]) * tmp);
        SWEEP(R_, FT[i] += ((D1Z(TT) * RO[i]) * p->DKAPA[z]) * tmp);
    }
    free(TTM);

    /* internal plume heat sink (iTCon 2), 3dmhdsub.h:443-459; RO holds 1/rho.
     * log(2.0f) is the float overload in the reference's C++ (3dmhdphsic.h
     * includes <math.h> before this code). */
    if (p->iTCon == 2) {
        const double CLN = (double)(-4.0f * logf(2.0f)) / p->HH / p->HH;
        const double s = (p->TC != 0.0)
                             ? p->TP * p->OCV * 0.5f * (1.0f + tanh((double)logf(2.0f) / p->QFH * (p->TIMT - p->TC)))
                             : p->TP * p->OCV;
        SWEEP(R_, FT[i] -= s * RO[i] * exp(CLN * sq(p->EXX[x] - p->XP) / p->HH) *
                           exp(CLN * sq(p->WYY[y] - p->YP) / p->HH) * exp(CLN * sq(p->ZEE[z] - p->ZP) / p->HH));
    }

    /* viscous Laplacians, 3dmhdsub.h:462-472 */
    SWEEP(R_, FU[i] += D2X(UU) * (p->ORE * p->C43));
    SWEEP(R_, FU[i] += D2Y(UU) * p->ORE);
    SWEEP(R_, FU[i] += D2Z(UU) * p->ORE);
    SWEEP(R_, FV[i] += D2X(VV) * p->ORE);
    SWEEP(R_, FV[i] += D2Y(VV) * (p->ORE * p->C43));
    SWEEP(R_, FV[i] += D2Z(VV) * p->ORE);
    SWEEP(R_, FW[i] += D2X(WW) * p->ORE);
    SWEEP(R_, FW[i] += D2Y(WW) * p->ORE);
    SWEEP(R_, FW[i] += D2Z(WW) * (p->ORE * p->C43));

    /* viscous cross terms, heating and pdV work, 3dmhdsub.h:475-538 */
    SWEEP(EXT_Y_, WW1[i] = D1X(UU));
    SWEEP(EXT_Y_, WW2[i] = D1X(VV));
    if (!p->lShr) {
        SWEEP(R_, WW3[i] = D1X(WW));
        tmp = p->OCV * p->ORE;
        SWEEP(R_, FT[i] += ((RO[i] * WW1[i]) * WW1[i]) * (tmp * p->C43));
        SWEEP(R_, FT[i] += ((RO[i] * WW2[i]) * WW2[i]) * tmp);
        SWEEP(R_, FT[i] += ((RO[i] * WW3[i]) * WW3[i]) * tmp);
        SWEEP(R_, FT[i] -= (WW1[i] * TT[i]) * p->OCV);
    }
    SWEEP(R_, FU[i] += D1Y(WW2) * (p->C13 * p->ORE));
    SWEEP(R_, FV[i] += D1Y(WW1) * (p->C13 * p->ORE));
    if (!p->lShr) {
        SWEEP(R_, WW1[i] = D1Y(UU));
        tmp = p->OCV * p->ORE;
        SWEEP(R_, FT[i] += ((RO[i] * WW1[i]) * WW1[i]) * tmp);
        SWEEP(R_, FT[i] += ((RO[i] * WW1[i]) * WW2[i]) * (tmp * 2));
        SWEEP(R_, WW2[i] = D1Y(VV));
        tmp = p->C43 * p->OCV * p->ORE;
        SWEEP(R_, FT[i] += ((RO[i] * WW2[i]) * WW2[i]) * tmp);
        SWEEP(R_, FT[i] -= (WW2[i] * TT[i]) * p->OCV);
        SWEEP(R_, WW1[i] = D1X(UU));
    }
    SWEEP(EXT_XY_, WW3[i] = D1Z(WW));
    if (!p->lShr) {
        tmp = p->C43 * p->OCV * p->ORE;
        SWEEP(R_, FT[i] += ((RO[i] * WW3[i]) * WW3[i]) * tmp);
        SWEEP(R_, FT[i] += ((RO[i] * WW1[i]) * WW3[i]) * (-tmp));
        SWEEP(R_, FT[i] += ((RO[i] * WW1[i]) * WW2[i]) * (-tmp));
        SWEEP(R_, FT[i] += ((RO[i] * WW2[i]) * WW3[i]) * (-tmp));
        SWEEP(R_, FT[i] -= (WW3[i] * TT[i]) * p->OCV);
    }
    SWEEP(R_, FU[i] += D1X(WW3) * (p->C13 * p->ORE));
    SWEEP(R_, FV[i] += D1Y(WW3) * (p->C13 * p->ORE));
    SWEEP(EXT_X_, WW1[i] = D1Z(UU));
    SWEEP(EXT_Y_, WW2[i] = D1Z(VV));
    if (!p->lShr) {
        SWEEP(R_, WW3[i] = D1Y(WW));
        tmp = p->OCV * p->ORE;
        SWEEP(R_, FT[i] += ((RO[i] * WW1[i]) * WW1[i]) * tmp);
        SWEEP(R_, FT[i] += ((RO[i] * WW2[i]) * WW2[i]) * tmp);
        SWEEP(R_, FT[i] += ((RO[i] * WW3[i]) * WW3[i]) * tmp);
        SWEEP(R_, FT[i] += ((RO[i] * WW2[i]) * WW3[i]) * (2.0f * tmp));
    }
    SWEEP(R_, FW[i] += D1X(WW1) * (p->C13 * p->ORE));
    SWEEP(R_, FW[i] += D1Y(WW2) * (p->C13 * p->ORE));
    if (!p->lShr) {
        SWEEP(R_, WW3[i] = D1X(WW));
        tmp = p->OCV * p->ORE;
        SWEEP(R_, FT[i] += ((RO[i] * WW1[i]) * WW3[i]) * (2.0f * tmp));
    }

    /* Coriolis, 3dmhdsub.h:540-545 */
    if (p->lRot) {
        SWEEP(R_, FU[i] += RV[i] * p->OMZ);
        SWEEP(R_, FV[i] -= RU[i] * p->OMZ);
        SWEEP(R_, FV[i] += RW[i] * p->OMX);
        SWEEP(R_, FW[i] -= RV[i] * p->OMX);
    }

    /* induction, Lorentz force and Ohmic heating, 3dmhdsub.h:547-695.
     * RU, RV, RW and TT are scratch from here on, as in the reference. */
    if (p->lMag) {
        const double c1 = p->OBETA * p->ORM * p->OCV;
        const double c2 = -2.0f * p->OBETA * p->ORM * p->OCV;
        SWEEP(R_, RU[i] = D1X(UU));
        SWEEP(R_, RV[i] = D1X(VV));
        SWEEP(R_, RW[i] = D1X(WW));
        SWEEP(R_, WW2[i] = BX[i] * RV[i]);
        SWEEP(R_, WW2[i] -= BY[i] * RU[i]);
        SWEEP(R_, WW3[i] = BX[i] * RW[i]);
        SWEEP(R_, WW3[i] -= BZ[i] * RU[i]);
        SWEEP(R_, RU[i] = D1Y(UU));
        SWEEP(R_, RV[i] = D1Y(VV));
        SWEEP(R_, RW[i] = D1Y(WW));
        SWEEP(R_, WW1[i] = BY[i] * RU[i]);
        SWEEP(R_, WW1[i] -= BX[i] * RV[i]);
        SWEEP(R_, WW3[i] += BY[i] * RW[i]);
        SWEEP(R_, WW3[i] -= BZ[i] * RV[i]);
        SWEEP(R_, RU[i] = D1Z(UU));
        SWEEP(R_, RV[i] = D1Z(VV));
        SWEEP(R_, RW[i] = D1Z(WW));
        /* one-sided dw/dz on the walls (3dmhdsub.h:572-584; each wall on its own rank) */
        SWEEP(zl, zl + 1, 1, ny - 1, 1, nx - 1,
              RW[i] = (4.0f * WW[i + sz] - WW[i + 2 * sz]) * p->hz * p->dzzdz[zl]);
        SWEEP(zr - 1, zr, 1, ny - 1, 1, nx - 1,
              RW[i] = (-4.0f * WW[i - sz] + WW[i - 2 * sz]) * p->hz * p->dzzdz[zr - 1]);
        SWEEP(R_, WW1[i] += BZ[i] * RU[i]);
        SWEEP(R_, WW1[i] -= BX[i] * RW[i]);
        SWEEP(R_, WW2[i] += BZ[i] * RV[i]);
        SWEEP(R_, WW2[i] -= BY[i] * RW[i]);
        SWEEP(R_, RU[i] = D1X(BX));
        SWEEP(R_, RV[i] = D1X(BY));
        SWEEP(R_, RW[i] = D1X(BZ));
        SWEEP(R_, TT[i] = D1Y(BX));
        SWEEP(R_, FU[i] += (BY[i] * TT[i]) * p->OBETA);
        SWEEP(R_, FU[i] -= (BY[i] * RV[i]) * p->OBETA);
        SWEEP(R_, FU[i] -= (BZ[i] * RW[i]) * p->OBETA);
        SWEEP(R_, FV[i] += (BX[i] * RV[i]) * p->OBETA);
        SWEEP(R_, FV[i] -= (BX[i] * TT[i]) * p->OBETA);
        SWEEP(R_, FW[i] += (BX[i] * RW[i]) * p->OBETA);
        SWEEP(R_, FT[i] += ((RO[i] * TT[i]) * TT[i]) * c1);
        SWEEP(R_, FT[i] += ((RO[i] * RV[i]) * RV[i]) * c1);
        SWEEP(R_, FT[i] += ((RO[i] * RW[i]) * RW[i]) * c1);
        SWEEP(R_, FT[i] += ((RO[i] * RV[i]) * TT[i]) * c2);
        SWEEP(R_, WW1[i] -= UU[i] * RU[i]);
        SWEEP(R_, WW1[i] -= VV[i] * TT[i]);
        SWEEP(R_, WW2[i] -= UU[i] * RV[i]);
        SWEEP(R_, WW3[i] -= UU[i] * RW[i]);
        SWEEP(R_, RU[i] = D2X(BX));
        SWEEP(R_, RV[i] = D2X(BY));
        SWEEP(R_, TT[i] = D2Y(BX));
        SWEEP(R_, WW1[i] += RU[i] * p->ORM);
        SWEEP(R_, WW1[i] += TT[i] * p->ORM);
        SWEEP(R_, WW2[i] += RV[i] * p->ORM);
        SWEEP(R_, TT[i] = D2X(BZ));
        SWEEP(R_, WW3[i] += TT[i] * p->ORM);
        SWEEP(R_, RU[i] = D1Z(BX));
        SWEEP(R_, RV[i] = D1Y(BY));
        SWEEP(R_, FU[i] += (BZ[i] * RU[i]) * p->OBETA);
        SWEEP(R_, FW[i] -= (BX[i] * RU[i]) * p->OBETA);
        SWEEP(R_, FT[i] += ((RO[i] * RU[i]) * RU[i]) * c1);
        SWEEP(R_, FT[i] += ((RO[i] * RU[i]) * RW[i]) * c2);
        SWEEP(R_, WW1[i] -= WW[i] * RU[i]);
        SWEEP(R_, WW2[i] -= VV[i] * RV[i]);
        SWEEP(R_, RU[i] = D2Z(BX));
        /* one-sided d2Bx/dz2 on the walls (3dmhdsub.h:640-654) */
        SWEEP(zl, zl + 1, 1, ny - 1, 1, nx - 1,
              RU[i] = (-3.0f * BX[i] + 4.0f * BX[i + sz] - BX[i + 2 * sz]) * p->hz * p->d2zzdz2[zl] +
                      (2.0f * BX[i] - 5.0f * BX[i + sz] + 4.0f * BX[i + 2 * sz] - BX[i + 3 * sz]) * p->h2z *
                          p->dzzdz[zl] * p->dzzdz[zl]);
        SWEEP(zr - 1, zr, 1, ny - 1, 1, nx - 1,
              RU[i] = (3.0f * BX[i] - 4.0f * BX[i - sz] + BX[i - 2 * sz]) * p->hz * p->d2zzdz2[zr - 1] +
                      (2.0f * BX[i] - 5.0f * BX[i - sz] + 4.0f * BX[i - 2 * sz] - BX[i - 3 * sz]) * p->h2z *
                          p->dzzdz[zr - 1] * p->dzzdz[zr - 1]);
        SWEEP(R_, RV[i] = D2Y(BY));
        SWEEP(R_, WW1[i] += RU[i] * p->ORM);
        SWEEP(R_, WW2[i] += RV[i] * p->ORM);
        SWEEP(R_, RV[i] = D1Z(BY));
        SWEEP(R_, RW[i] = D1Y(BZ));
        SWEEP(R_, RU[i] = RV[i]);
        SWEEP(R_, RU[i] -= RW[i]);
        SWEEP(R_, FV[i] += (BZ[i] * RU[i]) * p->OBETA);
        SWEEP(R_, FW[i] -= (BY[i] * RU[i]) * p->OBETA);
        SWEEP(R_, FT[i] += ((RO[i] * RV[i]) * RV[i]) * c1);
        SWEEP(R_, FT[i] += ((RO[i] * RW[i]) * RW[i]) * c1);
        SWEEP(R_, FT[i] += ((RO[i] * RV[i]) * RW[i]) * c2);
        SWEEP(R_, WW2[i] -= WW[i] * RV[i]);
        SWEEP(R_, WW3[i] -= VV[i] * RW[i]);
        SWEEP(R_, RV[i] = D2Z(BY));
        /* one-sided d2By/dz2 on the walls (3dmhdsub.h:673-687) */
        SWEEP(zl, zl + 1, 1, ny - 1, 1, nx - 1,
              RV[i] = (-3.0f * BY[i] + 4.0f * BY[i + sz] - BY[i + 2 * sz]) * p->hz * p->d2zzdz2[zl] +
                      (2.0f * BY[i] - 5.0f * BY[i + sz] + 4.0f * BY[i + 2 * sz] - BY[i + 3 * sz]) * p->h2z *
                          p->dzzdz[zl] * p->dzzdz[zl]);
        SWEEP(zr - 1, zr, 1, ny - 1, 1, nx - 1,
              RV[i] = (3.0f * BY[i] - 4.0f * BY[i - sz] + BY[i - 2 * sz]) * p->hz * p->d2zzdz2[zr - 1] +
                      (2.0f * BY[i] - 5.0f * BY[i - sz] + 4.0f * BY[i - 2 * sz] - BY[i - 3 * sz]) * p->h2z *
                          p->dzzdz[zr - 1] * p->dzzdz[zr - 1]);
        SWEEP(R_, RW[i] = D2Y(BZ));
        SWEEP(R_, WW2[i] += RV[i] * p->ORM);
        SWEEP(R_, WW3[i] += RW[i] * p->ORM);
        SWEEP(R_, RW[i] = D1Z(BZ));
        SWEEP(R_, WW3[i] -= WW[i] * RW[i]);
        SWEEP(R_, RW[i] = D2Z(BZ));
        SWEEP(R_, WW3[i] += RW[i] * p->ORM);
    }
    return 0;
}

/* step_block_ZETA0 / ZETA / GAM (3dmhdsub.h:155-192) with scale_add
 * tar = src1 + scale*srcd1 (3dmhdutils.h:57-59) */
void orc_rk_zeta0(const orc_params* p, orc_fields* f) {
    DECL_DIMS;
    set_threads(p);
    const int n = p->lMag ? 8 : 5;
    for (int k = 0; k < n; k++) {
        double* Z = f->a[ORC_ZRU + k];
        const double* U = f->a[ORC_RU + k];
        SWEEP(R_, Z[i] = U[i]);
    }
}

/* the F slot that drives each state slot: RU<-FU RV<-FV RW<-FW TT<-FT RO<-FR B<-WW1..3 */
static const int kFluxOf[8] = {ORC_FU, ORC_FV, ORC_FW, ORC_FT, ORC_FR, ORC_WW1, ORC_WW2, ORC_WW3};

void orc_rk_zeta(const orc_params* p, orc_fields* f, double coef) {
    DECL_DIMS;
    set_threads(p);
    const int n = p->lMag ? 8 : 5;
    for (int k = 0; k < n; k++) {
        double* Z = f->a[ORC_ZRU + k];
        const double* U = f->a[ORC_RU + k];
        const double* F = f->a[kFluxOf[k]];
        SWEEP(R_, Z[i] = U[i] + coef * F[i]);
    }
}

void orc_rk_gam(const orc_params* p, orc_fields* f, double coef) {
    DECL_DIMS;
    set_threads(p);
    const int n = p->lMag ? 8 : 5;
    for (int k = 0; k < n; k++) {
        double* U = f->a[ORC_RU + k];
        const double* Z = f->a[ORC_ZRU + k];
        const double* F = f->a[kFluxOf[k]];
        SWEEP(R_, U[i] = Z[i] + coef * F[i]);
    }
}

/* BCON, 3dmhdsub.h:720-873, both walls (the top on rank row myPEz==0, the
 * bottom on myPEz==nPEz-1 in the reference).  Returns -1 for the plume
 * variants (TP != 0 with iTCon 0/1) and for izCon outside {0,1}. */
int orc_bcon(const orc_params* p, orc_fields* f, double timt) {
    DECL_DIMS;
    double *RU = f->a[ORC_RU], *RV = f->a[ORC_RV], *RW = f->a[ORC_RW], *TT = f->a[ORC_TT], *RO = f->a[ORC_RO];
    double* BZ = f->a[ORC_BZ];
    const int zl = 1, zr = nz - 1;
    const double RRT = 1.0f, RRB = -1.0f, RPP = 0.0f;
    if (p->izCon != 0 && p->izCon != 1) return -1;
    if (p->iTCon != 0 && p->iTCon != 1 && p->iTCon != 2 && p->iTCon != 4) return -1;

    /* top wall */
    if (p->lShr) {
        SWEEP(zl, zl + 1, 1, ny - 1, 1, nx - 1, RU[i] = 0.0f; RV[i] = RRT * cos(RPP * timt) * RO[i]);
    } else {
        SWEEP(zl, zl + 1, 1, ny - 1, 1, nx - 1,
              RU[i] = RO[i] * (p->C43 * RU[i + sz] / RO[i + sz] - p->C13 * RU[i + 2 * sz] / RO[i + 2 * sz]);
              RV[i] = RO[i] * (p->C43 * RV[i + sz] / RO[i + sz] - p->C13 * RV[i + 2 * sz] / RO[i + 2 * sz]));
    }
    SWEEP(zl, zl + 1, 1, ny - 1, 1, nx - 1, RW[i] = 0.0f);
    if ((p->TP != 0.0) && (p->iTCon == 0 || p->iTCon == 1)) {
        /* cooling spot on the top wall, 3dmhdsub.h:750-778 */
        const double TPR = (p->TC != 0.0) ? p->TP + (1.0f - p->TP) * exp(-timt / p->TC) : p->TP;
        const double CLN = (double)(-4.0f * logf(2.0f)) / p->HH / p->HH;
        if (p->iTCon == 0) {
            SWEEP(zl, zl + 1, 1, ny - 1, 1, nx - 1,
                  TT[i] = 1.0f - (1.0f - TPR) * exp(CLN * sq(p->EXX[x] - p->XP)) / p->HH *
                                     exp(CLN * sq(p->WYY[y] - p->YP)) / p->HH);
        } else {
            const double DZ = 1.0f / (double)(p->nPz - 1) / p->dzzdz[zl];
            SWEEP(zl, zl + 1, 1, ny - 1, 1, nx - 1,
                  TT[i] = p->C43 * TT[i + sz] - p->C13 * TT[i + 2 * sz] -
                          p->C23 * DZ * (p->THETA - (p->THETA - TPR) * exp(CLN * sq(p->EXX[x] - p->XP)) / p->HH *
                                                        exp(CLN * sq(p->WYY[y] - p->YP)) / p->HH));
        }
    } else if (p->iTCon == 0 || p->iTCon == 2 || p->iTCon == 4) {
        const int is4 = p->iTCon == 4;
        if (p->lRem) {
            SWEEP(zl, zl + 1, 1, ny - 1, 1, nx - 1, TT[i] = p->TU);
        } else {
            SWEEP(zl, zl + 1, 1, ny - 1, 1, nx - 1, TT[i] = 1.0f; if (is4 && x < nx / 2) TT[i] = 1.0f - p->TP);
        }
    } else if (p->lRem) { /* iTCon == 1, lRem: 3dmhdsub.h:800-802 */
        SWEEP(zl, zl + 1, 1, ny - 1, 1, nx - 1, TT[i] = p->C43 * TT[i + sz] - p->C13 * TT[i + 2 * sz] + p->DZTU);
    } else { /* iTCon == 1 with TP == 0: fixed flux */
        const double DZ = 1.0f / (float)(p->nPz - 1) / p->dzzdz[zl];
        SWEEP(zl, zl + 1, 1, ny - 1, 1, nx - 1,
              TT[i] = p->C43 * TT[i + sz] - p->C13 * TT[i + 2 * sz] - p->C23 * DZ * p->THETA);
    }
    if (p->lMag && p->iBCon == 0) SWEEP(zl, zl + 1, 1, ny - 1, 1, nx - 1, BZ[i] = 0.0f);

    /* bottom wall */
    if (p->lShr) {
        SWEEP(zr - 1, zr, 1, ny - 1, 1, nx - 1, RU[i] = 0.0f; RV[i] = RRB * cos(RPP * timt) * RO[i]);
    } else {
        SWEEP(zr - 1, zr, 1, ny - 1, 1, nx - 1,
              RU[i] = RO[i] * (p->C43 * RU[i - sz] / RO[i - sz] - p->C13 * RU[i - 2 * sz] / RO[i - 2 * sz]);
              RV[i] = RO[i] * (p->C43 * RV[i - sz] / RO[i - sz] - p->C13 * RV[i - 2 * sz] / RO[i - 2 * sz]));
    }
    SWEEP(zr - 1, zr, 1, ny - 1, 1, nx - 1, RW[i] = 0.0f);
    if (p->izCon == 0) {
        SWEEP(zr - 1, zr, 1, ny - 1, 1, nx - 1, TT[i] = p->TB);
    } else if (p->lRem) { /* 3dmhdsub.h:852-854 */
        SWEEP(zr - 1, zr, 1, ny - 1, 1, nx - 1, TT[i] = p->C43 * TT[i - sz] - p->C13 * TT[i - 2 * sz] + p->DZTB);
    } else {
        const double DZ = 1.0f / (float)(p->nPz - 1) / p->dzzdz[zr - 1];
        SWEEP(zr - 1, zr, 1, ny - 1, 1, nx - 1,
              TT[i] = p->C43 * TT[i - sz] - p->C13 * TT[i - 2 * sz] - p->C23 * DZ * p->THETA / p->RKAPA[zr - 1]);
    }
    if (p->lMag && p->iBCon == 0) SWEEP(zr - 1, zr, 1, ny - 1, 1, nx - 1, BZ[i] = 0.0f);
    return 0;
}

/* communicate(), 3dmhdmpi.h:11-143, on one domain: every x/y ghost becomes the
 * periodic image; the z ghost planes are the walls' and stay as they are. */
void orc_communicate(const orc_params* p, orc_fields* f) {
    DECL_DIMS;
    static const int order[8] = {ORC_RU, ORC_RV, ORC_RW, ORC_TT, ORC_RO, ORC_BX, ORC_BY, ORC_BZ};
    const int n = p->lMag ? 8 : 5;
    for (int k = 0; k < n; k++) {
        double* V = f->a[order[k]];
        for (int z = 0; z < nz; z++) {
            double* pl = V + (size_t)z * sz;
            memcpy(pl, pl + (size_t)(ny - 2) * sy, sizeof(double) * (size_t)nx);
            memcpy(pl + (size_t)(ny - 1) * sy, pl + sy, sizeof(double) * (size_t)nx);
            for (int y = 0; y < ny; y++) {
                double* row = pl + (size_t)y * sy;
                row[0] = row[nx - 2];
                row[nx - 1] = row[1];
            }
        }
    }
}

static inline double dmin(double a, double b) { return (b < a) ? b : a; }
static inline double dmax(double a, double b) { return (a < b) ? b : a; }

/* CFL section of step(), 3dmhdsub.h:36-106 (ISW == 1) */
/* The CFL candidates of planes z in [z0, z1), folded in the reference's cell
 * order into r[0] = UMACH^2 max, r[1..4] = the four minima (3dmhdsub.h:36-106). */
static void cfl_planes(const orc_params* p, orc_fields* f, int z0, int z1, double r[5]) {
    DECL_DIMS;
    (void)nz;
    const double *RU = f->a[ORC_RU], *RV = f->a[ORC_RV], *RW = f->a[ORC_RW], *TT = f->a[ORC_TT], *RO = f->a[ORC_RO];
    const double *BX = f->a[ORC_BX], *BY = f->a[ORC_BY], *BZ = f->a[ORC_BZ];
    const double OGAMMA = 1.0f / p->GAMMA;
    double um = r[0], w0 = r[1], w1 = r[2], w2 = r[3], w3 = r[4];
    for (int z = z0; z < z1; z++)
        for (int y = 1; y < ny - 1; y++)
            for (int x = 1; x < nx - 1; x++) {
                const size_t i = ((size_t)z * ny + y) * nx + x;
                double UU = (RU[i] * RU[i] + RV[i] * RV[i] + RW[i] * RW[i]) / (RO[i] * RO[i]);
                um = dmax(um, OGAMMA * UU / TT[i]);
                if (p->lMag) {
                    UU += p->GAMMA * TT[i] + (BX[i] * BX[i] + BY[i] * BY[i] + BZ[i] * BZ[i]) * p->OBETA / RO[i] +
                          2.0f * sqrt(UU * (p->GAMMA * TT[i] + (BX[i] * BX[i] + BY[i] * BY[i] + BZ[i] * BZ[i]) * p->OBETA / RO[i]));
                } else {
                    UU += p->GAMMA * TT[i] + 2.0f * sqrt(p->GAMMA * UU * TT[i]);
                }
                double DD = dmin(p->DDY[y], p->DDZ[z]);
                if (nx > 3) DD = dmin(DD, p->DDX[x]);
                w0 = dmin(w0, DD / sqrt(UU));
                w1 = dmin(w1, p->lRem ? 0.5f * DD * DD * p->REPR * p->CV * RO[i] / (1.0f + p->RKAPA[z])
                                      : 0.5f * DD * DD * p->REPR * p->CV * RO[i] / p->RKAPA[z]);
                w2 = dmin(w2, 0.375f * DD * DD * p->RE * RO[i]);
                if (p->lMag) w3 = dmin(w3, 0.5f * DD * DD * p->RM);
            }
    r[0] = um; r[1] = w0; r[2] = w1; r[3] = w2; r[4] = w3;
}

double orc_cfl_dt(const orc_params* p, orc_fields* f, double* umach) {
    const int nz = p->nz;
    double r[5] = {0.0f, 1e99, 1e99, 1e99, 1e99};
    if (p->cfl_parallel) {
        /* every plane on its own thread from the neutral start, then folded in
         * plane order: min/max of finite values do not depend on the grouping */
        double* part = (double*)malloc(sizeof(double) * 5 * (size_t)nz);
        set_threads(p);
        ORC_PRAGMA(omp parallel for schedule(static))
        for (int z = 1; z < nz - 1; z++) {
            double* q = part + 5 * (size_t)z;
            q[0] = 0.0f; q[1] = q[2] = q[3] = q[4] = 1e99;
            cfl_planes(p, f, z, z + 1, q);
        }
        for (int z = 1; z < nz - 1; z++) {
            const double* q = part + 5 * (size_t)z;
            r[0] = dmax(r[0], q[0]);
            for (int k = 1; k < 5; k++) r[k] = dmin(r[k], q[k]);
        }
        free(part);
    } else {
        cfl_planes(p, f, 1, nz - 1, r);
    }
    if (umach) *umach = sqrt(r[0]);
    if (p->lMag) return p->SFF * dmin(dmin(r[1], r[2]), dmin(r[3], r[4]));
    return p->SFF * dmin(dmin(r[1], r[2]), r[3]);
}

int orc_steps(const orc_params* p0, orc_fields* f, int n, double dt, double* timt, double* dt_out) {
    orc_params q = *p0;  /* fluxes() sees the step's TIMT */
    const orc_params* p = &q;
    double t = timt ? *timt : 0.0;
    const double timi = t;
    double timc = 0.0;
    for (int s = 0; s < n; s++) {
        double DT = dt;
        if (dt <= 0.0) DT = orc_cfl_dt(p, f, NULL);
        q.TIMT = t;
        orc_rk_zeta0(p, f);
        orc_fluxes(p, f);
        orc_rk_gam(p, f, p->GAM1 * DT);
        if (orc_bcon(p, f, t)) return -1;
        orc_communicate(p, f);
        orc_rk_zeta(p, f, p->ZETA1 * DT);
        orc_fluxes(p, f);
        orc_rk_gam(p, f, p->GAM2 * DT);
        if (orc_bcon(p, f, t)) return -1;
        orc_communicate(p, f);
        orc_rk_zeta(p, f, p->ZETA2 * DT);
        orc_fluxes(p, f);
        orc_rk_gam(p, f, p->GAM3 * DT);
        if (orc_bcon(p, f, t)) return -1;
        orc_communicate(p, f);
        timc += DT;
        t = timi + timc;
        if (dt_out) dt_out[s] = DT;
    }
    if (timt) *timt = t;
    return 0;
}
