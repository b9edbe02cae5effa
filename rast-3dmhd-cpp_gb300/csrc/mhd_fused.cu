// mhd_fused.cu -- one fused pass per Wray RK3 substage, FP64.
//
// Each CTA owns a TX x TY tile of (x, y) columns and marches down z.  Three
// z-planes of the tile plus a one-cell halo live in a shared-memory ring;
// when plane z+2 is loaded its derived quantities (1/rho, the velocities
// u = RU/rho, v, w and the pressure p = rho*T) are computed once per point,
// so every stencil below reads them instead of recomputing them.  One
// thread per column then evaluates the whole right-hand side of fluxes()
// (3dmhdsub.h:194-696) for cell (z, y, x), applies the RK update of
// step_block_GAM (3dmhdsub.h:181-192), forms the next substage's register
// Z' = U' + zeta*dt*F (step_block_ZETA, 3dmhdsub.h:168-179) and writes U'
// together with its periodic ghost images (communicate(), 3dmhdmpi.h:11-143,
// as dual stores).  A small kernel then applies BCON (3dmhdsub.h:720-873) to
// the two wall planes of U' and refreshes their ghost images.
//
// The right-hand side is the reference's, regrouped to use the fewest FP64
// instructions (GB300's FP64 rate, not HBM, bounds this kernel): metric
// factors are premultiplied (c1 = duudu*hu, c2a = d2uudu2*hu,
// c2b = duudu^2*h2u), repeated gradients are computed once, and sums of
// products use FMA.  Results agree with the reference to rounding
// (checked against the oracle at 1e-12 of each field's max-norm).
//
// Wall planes: the values the reference overwrites in BCON (RU, RV, RW, TT,
// BZ and, with lShr, the right-hand side FT) are finite but not the
// reference's before BCON runs; RO, BX, BY and everything on interior planes
// follow the reference.  The z ghost planes are never written (the reference
// only flips RO there between rho and 1/rho; those values reach no result).
#include "mhd_common.cuh"

namespace mhd {
namespace {

constexpr int kTX = 32;
constexpr int kTY = 4;
constexpr int kThreads = kTX * kTY;
constexpr int kPX = kTX + 2;
constexpr int kPY = kTY + 2;
constexpr int kPlane = kPX * kPY;

// quantities held per plane point
enum Q { Q_RU = 0, Q_RV, Q_RW, Q_TT, Q_RO, Q_RI, Q_U, Q_V, Q_W, Q_P, Q_BX, Q_BY, Q_BZ, Q_N };

template <class SW>
constexpr int nq() {
    return SW::lMag ? Q_N : Q_BX;
}

template <class SW>
__device__ __forceinline__ void load_plane(const FusedArgs& a, double* ring, int slot, int z, int x0, int y0) {
    constexpr int NQ = nq<SW>();
    double* base = ring + (size_t)slot * NQ * kPlane;
    const Grid& g = a.g;
    for (int k = threadIdx.x; k < kPlane; k += kThreads) {
        const int hx = k % kPX, hy = k / kPX;
        const int gx = x0 - 1 + hx, gy = y0 - 1 + hy;
        if (gx >= g.nx || gy >= g.ny) continue;
        const long long i = (long long)z * g.sz + (long long)gy * g.sy + gx;
        const double ru = a.U.p[S_RU][i], rv = a.U.p[S_RV][i], rw = a.U.p[S_RW][i];
        const double tt = a.U.p[S_TT][i], ro = a.U.p[S_RO][i];
        const double ri = 1.0 / ro;
        base[Q_RU * kPlane + k] = ru;
        base[Q_RV * kPlane + k] = rv;
        base[Q_RW * kPlane + k] = rw;
        base[Q_TT * kPlane + k] = tt;
        base[Q_RO * kPlane + k] = ro;
        base[Q_RI * kPlane + k] = ri;
        base[Q_U * kPlane + k] = ru * ri;
        base[Q_V * kPlane + k] = rv * ri;
        base[Q_W * kPlane + k] = rw * ri;
        base[Q_P * kPlane + k] = ro * tt;
        if constexpr (SW::lMag) {
            base[Q_BX * kPlane + k] = a.U.p[S_BX][i];
            base[Q_BY * kPlane + k] = a.U.p[S_BY][i];
            base[Q_BZ * kPlane + k] = a.U.p[S_BZ][i];
        }
    }
}

// Store v at (z, y, x) and at every periodic ghost image of that cell.
__device__ __forceinline__ void store_with_images(double* F, const Grid& g, int z, int y, int x, double v) {
    const long long zo = (long long)z * g.sz;
    const int ya = y, xa = x;
    const int yb = (y == 1) ? g.ny - 1 : (y == g.ny - 2 ? 0 : -1);
    const int xb = (x == 1) ? g.nx - 1 : (x == g.nx - 2 ? 0 : -1);
    F[zo + (long long)ya * g.sy + xa] = v;
    if (xb >= 0) F[zo + (long long)ya * g.sy + xb] = v;
    if (yb >= 0) {
        F[zo + (long long)yb * g.sy + xa] = v;
        if (xb >= 0) F[zo + (long long)yb * g.sy + xb] = v;
    }
}

template <class SW>
__global__ void __launch_bounds__(kThreads) k_substage(FusedArgs a) {
    constexpr int NQ = nq<SW>();
    extern __shared__ double ring[];
    const Grid& g = a.g;
    const Consts& c = a.c;
    const int x0 = 1 + blockIdx.x * kTX, y0 = 1 + blockIdx.y * kTY;
    const int tx = threadIdx.x % kTX, ty = threadIdx.x / kTX;
    const int x = x0 + tx, y = y0 + ty;
    const bool active = (x <= g.nx - 2) && (y <= g.ny - 2);
    const int zl = 1, zr = g.nz - 1;

    // per-column metric coefficients
    const int xc = active ? x : 1, yc = active ? y : 1;
    const double cx1 = a.k.cx1[xc], cx2a = a.k.cx2a[xc], cx2b = a.k.cx2b[xc];
    const double cy1 = a.k.cy1[yc], cy2a = a.k.cy2a[yc], cy2b = a.k.cy2b[yc];
    const double c13ore = c.C13 * c.ORE;
    const double kxy = c13ore * cx1 * cy1;
    const double ore43 = c.ORE * c.C43;
    const double ocvore = c.OCV * c.ORE;
    const double ohm = c.OBETA * c.ORM * c.OCV;
    const double tmpc = c.OCV / c.REPR;

    load_plane<SW>(a, ring, 0, 0, x0, y0);
    load_plane<SW>(a, ring, 1, 1, x0, y0);
    load_plane<SW>(a, ring, 2, 2, x0, y0);

    const int pc = (ty + 1) * kPX + (tx + 1);  // centre offset inside a plane
    for (int z = 1; z <= g.nz - 2; z++) {
        __syncthreads();
        if (active) {
            const double* Pm = ring + (size_t)((z - 1) % 3) * NQ * kPlane;
            const double* P0 = ring + (size_t)(z % 3) * NQ * kPlane;
            const double* Pp = ring + (size_t)((z + 1) % 3) * NQ * kPlane;
            auto C0 = [&](int q) { return P0[q * kPlane + pc]; };
            auto XP = [&](int q) { return P0[q * kPlane + pc + 1]; };
            auto XM = [&](int q) { return P0[q * kPlane + pc - 1]; };
            auto YP = [&](int q) { return P0[q * kPlane + pc + kPX]; };
            auto YM = [&](int q) { return P0[q * kPlane + pc - kPX]; };
            auto ZP = [&](int q) { return Pp[q * kPlane + pc]; };
            auto ZM = [&](int q) { return Pm[q * kPlane + pc]; };
            const double cz1 = a.k.cz1[z], cz2a = a.k.cz2a[z], cz2b = a.k.cz2b[z];
            auto Dx = [&](int q) { return (XP(q) - XM(q)) * cx1; };
            auto Dy = [&](int q) { return (YP(q) - YM(q)) * cy1; };
            auto Dz = [&](int q) { return (ZP(q) - ZM(q)) * cz1; };
            // second derivatives scaled by s: s*D2 = (dF*c2a + d2F*c2b)*s
            auto D2x = [&](int q) {
                const double p = XP(q), m = XM(q);
                return fma(p - m, cx2a, fma(-2.0, C0(q), p + m) * cx2b);
            };
            auto D2y = [&](int q) {
                const double p = YP(q), m = YM(q);
                return fma(p - m, cy2a, fma(-2.0, C0(q), p + m) * cy2b);
            };
            auto D2z = [&](int q) {
                const double p = ZP(q), m = ZM(q);
                return fma(p - m, cz2a, fma(-2.0, C0(q), p + m) * cz2b);
            };

            const double ro = C0(Q_RO), ri = C0(Q_RI), tt = C0(Q_TT);
            const double u = C0(Q_U), v = C0(Q_V), w = C0(Q_W);
            const long long i = (long long)z * g.sz + (long long)y * g.sy + x;

            // ---- continuity (3dmhdsub.h:204-227), one-sided dRW/dz on walls
            double rwz = Dz(Q_RW);
            if (z == zl) rwz = (4.0 * ZP(Q_RW) - a.U.p[S_RW][i + 2 * g.sz]) * cz1;
            if (z == zr - 1) rwz = (a.U.p[S_RW][i - 2 * g.sz] - 4.0 * ZM(Q_RW)) * cz1;
            const double fr = -(Dx(Q_RU) + Dy(Q_RV) + rwz);

            // ---- pressure and gravity (3dmhdsub.h:266-272)
            double fu = -Dx(Q_P);
            double fv = -Dy(Q_P);
            double fw = fma(ro, c.GRAV, -Dz(Q_P));

            // ---- momentum advection (3dmhdsub.h:279-289): -D_j(RU_i u_j)
            fu -= fma(XP(Q_RU), XP(Q_U), -XM(Q_RU) * XM(Q_U)) * cx1;
            fu -= fma(YP(Q_RU), YP(Q_V), -YM(Q_RU) * YM(Q_V)) * cy1;
            fu -= fma(ZP(Q_RU), ZP(Q_W), -ZM(Q_RU) * ZM(Q_W)) * cz1;
            fv -= fma(XP(Q_RV), XP(Q_U), -XM(Q_RV) * XM(Q_U)) * cx1;
            fv -= fma(YP(Q_RV), YP(Q_V), -YM(Q_RV) * YM(Q_V)) * cy1;
            fv -= fma(ZP(Q_RV), ZP(Q_W), -ZM(Q_RV) * ZM(Q_W)) * cz1;
            fw -= fma(XP(Q_RW), XP(Q_U), -XM(Q_RW) * XM(Q_U)) * cx1;
            fw -= fma(YP(Q_RW), YP(Q_V), -YM(Q_RW) * YM(Q_V)) * cy1;
            fw -= fma(ZP(Q_RW), ZP(Q_W), -ZM(Q_RW) * ZM(Q_W)) * cz1;

            // ---- temperature: advection (3dmhdsub.h:293-296) and conduction (:315-319)
            const double Tz = Dz(Q_TT);
            double ft;
            if constexpr (!SW::lShr) {
                ft = -fma(u, Dx(Q_TT), fma(v, Dy(Q_TT), w * Tz));
            } else {
                ft = a.FT[i];  // the reference never re-initialises FT with lShr
            }
            {
                const double lapT = D2x(Q_TT) + D2y(Q_TT) + D2z(Q_TT);
                ft = fma(ri * tmpc, fma(c.RKAPA[z], lapT, c.DKAPA[z] * Tz), ft);
            }

            // ---- viscous Laplacians (3dmhdsub.h:462-472)
            fu = fma(ore43, D2x(Q_U), fma(c.ORE, D2y(Q_U) + D2z(Q_U), fu));
            fv = fma(ore43, D2y(Q_V), fma(c.ORE, D2x(Q_V) + D2z(Q_V), fv));
            fw = fma(ore43, D2z(Q_W), fma(c.ORE, D2x(Q_W) + D2y(Q_W), fw));

            // ---- viscous cross terms (3dmhdsub.h:486-487,517-518,531-532)
            {
                const double kxz = c13ore * cx1 * cz1, kyz = c13ore * cy1 * cz1;
                auto E = [&](const double* Pl, int q, int off) { return Pl[q * kPlane + pc + off]; };
                // D_y D_x v, D_y D_x u
                const double dyxv = (E(P0, Q_V, kPX + 1) - E(P0, Q_V, kPX - 1)) - (E(P0, Q_V, -kPX + 1) - E(P0, Q_V, -kPX - 1));
                const double dyxu = (E(P0, Q_U, kPX + 1) - E(P0, Q_U, kPX - 1)) - (E(P0, Q_U, -kPX + 1) - E(P0, Q_U, -kPX - 1));
                // D_x D_z w, D_y D_z w
                const double dxzw = (E(Pp, Q_W, 1) - E(Pm, Q_W, 1)) - (E(Pp, Q_W, -1) - E(Pm, Q_W, -1));
                const double dyzw = (E(Pp, Q_W, kPX) - E(Pm, Q_W, kPX)) - (E(Pp, Q_W, -kPX) - E(Pm, Q_W, -kPX));
                // D_x D_z u, D_y D_z v
                const double dxzu = (E(Pp, Q_U, 1) - E(Pm, Q_U, 1)) - (E(Pp, Q_U, -1) - E(Pm, Q_U, -1));
                const double dyzv = (E(Pp, Q_V, kPX) - E(Pm, Q_V, kPX)) - (E(Pp, Q_V, -kPX) - E(Pm, Q_V, -kPX));
                fu = fma(kxy, dyxv, fma(kxz, dxzw, fu));
                fv = fma(kxy, dyxu, fma(kyz, dyzw, fv));
                fw = fma(kxz, dxzu, fma(kyz, dyzv, fw));
            }

            // velocity gradients (heating and induction)
            double ux = 0, uy = 0, uz = 0, vx = 0, vy = 0, vz = 0, wx = 0, wy = 0, wz = 0;
            if constexpr (!SW::lShr || SW::lMag) {
                ux = Dx(Q_U); uy = Dy(Q_U); uz = Dz(Q_U);
                vx = Dx(Q_V); vy = Dy(Q_V); vz = Dz(Q_V);
                wx = Dx(Q_W); wy = Dy(Q_W); wz = Dz(Q_W);
            }
            // ---- viscous heating and pdV work (3dmhdsub.h:477-538, not with lShr)
            if constexpr (!SW::lShr) {
                double dg = ux * ux;
                dg = fma(vy, vy, dg);
                dg = fma(wz, wz, dg);
                dg = fma(-ux, vy, dg);
                dg = fma(-ux, wz, dg);
                dg = fma(-vy, wz, dg);
                const double s1 = uy + vx, s2 = uz + wx, s3 = vz + wy;
                const double sh = fma(s1, s1, fma(s2, s2, s3 * s3));
                const double phi = fma(c.C43, dg, sh);
                ft = fma(ocvore * ri, phi, ft);
                ft = fma(-c.OCV * tt, ux + vy + wz, ft);
            }

            // ---- Coriolis (3dmhdsub.h:540-545)
            if constexpr (SW::lRot) {
                fu = fma(c.OMZ, C0(Q_RV), fu);
                fv = fma(-c.OMZ, C0(Q_RU), fv);
                fv = fma(c.OMX, C0(Q_RW), fv);
                fw = fma(-c.OMX, C0(Q_RV), fw);
            }

            // ---- induction, Lorentz force, Ohmic heating (3dmhdsub.h:547-695)
            double w1 = 0, w2 = 0, w3 = 0;
            if constexpr (SW::lMag) {
                const double bx = C0(Q_BX), by = C0(Q_BY), bz = C0(Q_BZ);
                // one-sided dw/dz on the walls for the induction terms (3dmhdsub.h:572-584)
                double wzm = wz;
                if (z == zl) {
                    const long long j = i + 2 * g.sz;
                    wzm = (4.0 * ZP(Q_W) - a.U.p[S_RW][j] / a.U.p[S_RO][j]) * cz1;
                }
                if (z == zr - 1) {
                    const long long j = i - 2 * g.sz;
                    wzm = (a.U.p[S_RW][j] / a.U.p[S_RO][j] - 4.0 * ZM(Q_W)) * cz1;
                }
                const double bxx = Dx(Q_BX), bxy = Dy(Q_BX), bxz = Dz(Q_BX);
                const double byx = Dx(Q_BY), byy = Dy(Q_BY), byz = Dz(Q_BY);
                const double bzx = Dx(Q_BZ), bzy = Dy(Q_BZ), bzz = Dz(Q_BZ);
                double lbx = D2x(Q_BX) + D2y(Q_BX);
                double lby = D2x(Q_BY) + D2y(Q_BY);
                const double lbz = D2x(Q_BZ) + D2y(Q_BZ) + D2z(Q_BZ);
                // d2B/dz2 with the one-sided wall stencils (3dmhdsub.h:640-654,673-687)
                if (z == zl || z == zr - 1) {
                    const int s = (z == zl) ? 1 : -1;
                    const long long j2 = i + 2 * s * g.sz, j3 = i + 3 * s * g.sz;
                    const double d2 = c.d2zzdz2[z] * c.hz, d1 = c.dzzdz[z] * c.dzzdz[z] * c.h2z;
                    const double X0 = bx, X1 = (s > 0) ? ZP(Q_BX) : ZM(Q_BX);
                    const double X2 = a.U.p[S_BX][j2], X3 = a.U.p[S_BX][j3];
                    const double Y0 = by, Y1 = (s > 0) ? ZP(Q_BY) : ZM(Q_BY);
                    const double Y2 = a.U.p[S_BY][j2], Y3 = a.U.p[S_BY][j3];
                    const double sg = (double)s;
                    lbx += sg * (-3.0 * X0 + 4.0 * X1 - X2) * d2 + (2.0 * X0 - 5.0 * X1 + 4.0 * X2 - X3) * d1;
                    lby += sg * (-3.0 * Y0 + 4.0 * Y1 - Y2) * d2 + (2.0 * Y0 - 5.0 * Y1 + 4.0 * Y2 - Y3) * d1;
                } else {
                    lbx += D2z(Q_BX);
                    lby += D2z(Q_BY);
                }
                w1 = fma(by, uy, fma(bz, uz, -bx * (vy + wzm)));
                w1 = fma(-u, bxx, fma(-v, bxy, fma(-w, bxz, w1)));
                w1 = fma(c.ORM, lbx, w1);
                w2 = fma(bx, vx, fma(bz, vz, -by * (ux + wzm)));
                w2 = fma(-u, byx, fma(-v, byy, fma(-w, byz, w2)));
                w2 = fma(c.ORM, lby, w2);
                w3 = fma(bx, wx, fma(by, wy, -bz * (ux + vy)));
                w3 = fma(-u, bzx, fma(-v, bzy, fma(-w, bzz, w3)));
                w3 = fma(c.ORM, lbz, w3);
                const double jz = byx - bxy, jy = bxz - bzx, jx = bzy - byz;
                fu = fma(c.OBETA, fma(bz, jy, -by * jz), fu);
                fv = fma(c.OBETA, fma(bx, jz, -bz * jx), fv);
                fw = fma(c.OBETA, fma(by, jx, -bx * jy), fw);
                ft = fma(ohm * ri, fma(jx, jx, fma(jy, jy, jz * jz)), ft);
            }

            // ---- RK3 substage update and the next register (3dmhdsub.h:168-192)
            const double fl[8] = {fu, fv, fw, ft, fr, w1, w2, w3};
            const int nf = SW::lMag ? 8 : 5;
            const double cen[8] = {C0(Q_RU), C0(Q_RV), C0(Q_RW), tt, ro,
                                   SW::lMag ? C0(Q_BX < NQ ? Q_BX : 0) : 0.0,
                                   SW::lMag ? C0(Q_BY < NQ ? Q_BY : 0) : 0.0,
                                   SW::lMag ? C0(Q_BZ < NQ ? Q_BZ : 0) : 0.0};
#pragma unroll
            for (int f = 0; f < 8; f++) {
                if (f >= nf) break;
                const double zf = (a.substage == 0) ? cen[f] : a.Z.p[f][i];
                const double un = fma(a.gdt, fl[f], zf);
                store_with_images(a.Uo.p[f], g, z, y, x, un);
                if (a.substage < 2) a.Z.p[f][i] = fma(a.zdt, fl[f], un);
            }
            if constexpr (SW::lShr) a.FT[i] = ft;
        }
        __syncthreads();
        if (z + 2 <= g.nz - 1) load_plane<SW>(a, ring, (z + 2) % 3, z + 2, x0, y0);
    }
}

// BCON on the two wall planes of U' plus their periodic ghost images.
template <class SW>
__global__ void k_bcon_ghost(Grid g, Consts c, Fields8 U, double timt) {
    const int nPx = g.nx - 2, nPy = g.ny - 2;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 2 * nPx * nPy) return;
    const int wall = t / (nPx * nPy);
    const int r = t % (nPx * nPy);
    const int x = 1 + r % nPx, y = 1 + r / nPx;
    const long long sz = g.sz;
    const double RRT = 1.0, RRB = -1.0, RPP = 0.0;
    const int z = wall == 0 ? 1 : g.nz - 2;
    const int s = wall == 0 ? 1 : -1;
    const long long i = (long long)z * sz + (long long)y * g.sy + x;
    const long long i1 = i + s * sz, i2 = i + 2 * s * sz;
    double *RU = U.p[S_RU], *RV = U.p[S_RV], *TT = U.p[S_TT];
    const double* RO = U.p[S_RO];
    double ru, rv, tt;
    if constexpr (SW::lShr) {
        ru = 0.0;
        rv = (wall == 0 ? RRT : RRB) * cos(RPP * timt) * RO[i];
    } else {
        ru = RO[i] * (c.C43 * RU[i1] / RO[i1] - c.C13 * RU[i2] / RO[i2]);
        rv = RO[i] * (c.C43 * RV[i1] / RO[i1] - c.C13 * RV[i2] / RO[i2]);
    }
    if (wall == 0) {
        if (c.iTCon == 1) {
            const double DZ = 1.0f / (float)(g.nPz - 1) / c.dzzdz[z];
            tt = c.C43 * TT[i1] - c.C13 * TT[i2] - c.C23 * DZ * c.THETA;
        } else {
            tt = 1.0;
            if (c.iTCon == 4 && x < g.nx / 2) tt = 1.0f - c.TP;
        }
    } else {
        if (c.izCon == 0) {
            tt = c.TB;
        } else {
            const double DZ = 1.0f / (float)(g.nPz - 1) / c.dzzdz[z];
            tt = c.C43 * TT[i1] - c.C13 * TT[i2] - c.C23 * DZ * c.THETA / c.RKAPA[z];
        }
    }
    store_with_images(U.p[S_RU], g, z, y, x, ru);
    store_with_images(U.p[S_RV], g, z, y, x, rv);
    store_with_images(U.p[S_RW], g, z, y, x, 0.0);
    store_with_images(U.p[S_TT], g, z, y, x, tt);
    if constexpr (SW::lMag) {
        if (c.iBCon == 0) store_with_images(U.p[S_BZ], g, z, y, x, 0.0);
    }
}

template <class SW>
void launch_substage(const FusedArgs& a, cudaStream_t st, int* rc) {
    const size_t smem = (size_t)3 * nq<SW>() * kPlane * sizeof(double);
    static bool configured = false;
    if (!configured) {
        cudaFuncSetAttribute(k_substage<SW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        configured = true;
    }
    const dim3 grid((a.g.nx - 2 + kTX - 1) / kTX, (a.g.ny - 2 + kTY - 1) / kTY);
    k_substage<SW><<<grid, kThreads, smem, st>>>(a);
    *rc = (int)cudaGetLastError();
}

template <class SW>
void launch_bcon_ghost(const Grid& g, const Consts& c, Fields8 U, double timt, cudaStream_t st) {
    const int n = 2 * (g.nx - 2) * (g.ny - 2);
    k_bcon_ghost<SW><<<(n + 127) / 128, 128, 0, st>>>(g, c, U, timt);
}

}  // namespace

int fused_substage(unsigned sw, const FusedArgs& a, cudaStream_t st) {
    int rc = 0;
    MHD_DISPATCH_SW(sw, launch_substage, a, st, &rc);
    return rc;
}

int fused_bcon_ghost(unsigned sw, const Grid& g, const Consts& c, Fields8 U, double timt, cudaStream_t st) {
    MHD_DISPATCH_SW(sw, launch_bcon_ghost, g, c, U, timt, st);
    return (int)cudaGetLastError();
}

}  // namespace mhd
