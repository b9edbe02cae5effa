/*
 * mhd_oracle.h -- CPU restatement of the reference 3dmhd hot path on one
 * global domain.  TEST INFRASTRUCTURE: used only by tests/, the smoke check
 * and the CPU-baseline leg of bench.py, as the checker.  It is never on the
 * product path.
 *
 * Every routine follows the reference's sweep order and expression
 * association so that, compiled with -ffp-contract=off, it reproduces the
 * reference bit for bit (pinned by tests/test_oracle_golden.py against
 * fixtures produced by the reference itself).
 */
#ifndef MHD_ORACLE_H_
#define MHD_ORACLE_H_

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_params {
    int nx, ny, nz;      /* full array sizes including the 1-cell ghosts */
    int nPz;             /* interior z points (3dmhdparam.h:27) */
    int lMag, lRot, lShr;
    int izCon, iTCon, iBCon;
    int nthreads;        /* OpenMP threads, <=0 leaves the runtime default */
    int cfl_parallel;    /* 1: orc_cfl_dt reduces planes on all threads (the same
                            result for finite states; with NaN/Inf only the default
                            serial order is the reference's) -- timing runs only */
    /* scalars as set() and main() leave them (3dmhd.cpp:144-145,354-369,401-459) */
    double C13, C23, C43, GAM1, GAM2, GAM3, ZETA1, ZETA2;
    double hx, h2x, hy, h2y, hz, h2z;
    double RE, PR, REPR, ORE, CV, OCV, GAMMA, GRAV, THETA;
    double RY, ANG, OMX, OMZ, RM, ORM, BETA, OBETA, TB, TP, SFF;
    /* 1-D metric arrays: x has nx entries, y ny, z nz (3dmhddata.h:21-23) */
    const double *dxxdx, *d2xxdx2, *DDX;
    const double *dyydy, *d2yydy2, *DDY;
    const double *dzzdz, *d2zzdz2, *DDZ;
    const double *RKAPA, *DKAPA;
    /* plume terms (3dmhdsub.h:443-459,750-778): coordinates (x nx, y ny, z nz
     * entries; may be NULL when no plume term is active), parameters
     * (3dmhd.cpp:413-426) and the simulation time TIMT the source sees */
    const double *EXX, *WYY, *ZEE;
    double XP, YP, ZP, HH, TC, QFH;
    double TIMT;
    /* lRem (Rempel relaxation; 3dmhdsub.h:229-242,297-313,783-802,852-854):
     * switch and the static model's TU, DZTU, DZTB (3dmhdphsic.h:592-594) */
    int lRem, pad2_;
    double TU, DZTU, DZTB;
} orc_params;

/* Field slots.  0-7 state, 8-15 right-hand sides, 16-23 RK register,
 * 24-26 velocity scratch.  Every pointer addresses nz*ny*nx doubles. */
enum {
    ORC_RU = 0, ORC_RV, ORC_RW, ORC_TT, ORC_RO, ORC_BX, ORC_BY, ORC_BZ,
    ORC_FU, ORC_FV, ORC_FW, ORC_FR, ORC_FT, ORC_WW1, ORC_WW2, ORC_WW3,
    ORC_ZRU, ORC_ZRV, ORC_ZRW, ORC_ZTT, ORC_ZRO, ORC_ZBX, ORC_ZBY, ORC_ZBZ,
    ORC_UU, ORC_VV, ORC_WW, ORC_NSLOTS
};

typedef struct orc_fields {
    double* a[ORC_NSLOTS];
} orc_fields;

/* Fill the derived scalars from RE, PR, THETA, GRAV, RY, ANG, RM, BETA,
 * GAMMA, TB, TP, SFF and the grid size, exactly as set() does. */
void orc_set_constants(orc_params* p, int nPx, int nPy, int nPz);

int orc_fluxes(const orc_params* p, orc_fields* f);                  /* 3dmhdsub.h:194-696 */
void orc_rk_zeta0(const orc_params* p, orc_fields* f);               /* 3dmhdsub.h:155-166 */
void orc_rk_zeta(const orc_params* p, orc_fields* f, double coef);   /* 3dmhdsub.h:168-179 */
void orc_rk_gam(const orc_params* p, orc_fields* f, double coef);    /* 3dmhdsub.h:181-192 */
int orc_bcon(const orc_params* p, orc_fields* f, double timt);       /* 3dmhdsub.h:720-873 */
void orc_communicate(const orc_params* p, orc_fields* f);            /* 3dmhdmpi.h:11-143 */
/* CFL time step of step() (3dmhdsub.h:36-106); also returns UMACH. */
double orc_cfl_dt(const orc_params* p, orc_fields* f, double* umach);
/* n RK3 steps (3dmhdsub.h:116-152).  dt > 0: fixed step; dt <= 0: CFL step
 * each iteration.  *timt advances like TIMT; dt_out (may be NULL) gets each
 * step's DT. */
int orc_steps(const orc_params* p, orc_fields* f, int n, double dt, double* timt, double* dt_out);

#ifdef __cplusplus
}
#endif

#endif
