// mhd_fused_tile.cuh -- the fused FP64 RK3 substage for one tile of columns.
//
// A CTA owns a TX x TY tile of (x, y) columns and marches down a range of z
// planes.  Three z-planes of the tile plus a one-cell halo live in a
// shared-memory ring; when plane z+2 is loaded its derived quantities (1/rho,
// the velocities u = RU/rho, v, w and the diagonal momentum fluxes
// p + RU u, p + RV v, p + RW w with the pressure p = rho*T) are computed once
// per point, so every stencil reads them instead of recomputing them.
// One thread per column then evaluates the whole right-hand side of fluxes()
// (3dmhdsub.h:194-696) for cell (z, y, x), applies the RK update of
// step_block_GAM (3dmhdsub.h:181-192), forms the next substage's register
// Z' = U' + zeta*dt*F (step_block_ZETA, 3dmhdsub.h:168-179) and writes U'
// together with its periodic ghost images (communicate(), 3dmhdmpi.h:11-143,
// as dual stores).  BCON (3dmhdsub.h:720-873) on the wall planes follows in a
// separate small kernel.
//
// GB300 executes two FP64 FMAs per clock per SM, so this kernel is bound by
// its FP64 instruction count, not by HBM; the right-hand side is regrouped for
// the fewest FP64 instructions:
//   * metric factors are premultiplied (c1 = duudu*hu, c2a = d2uudu2*hu,
//     c2b = duudu^2*h2u), and the viscous (ORE, ORE*C43) and resistive (ORM)
//     scales are folded into copies of c2a/c2b, so a scaled second derivative
//     accumulates with three FMAs (five where d2uudu2 does not vanish);
//   * UXY (uniform x and y grids: d2uudu2 = 0, the same coefficients in
//     every column) drops the first-derivative part of the x/y second
//     derivatives at compile time and sums each Laplacian as
//     sx (px + mx) + sy (py + my) + pz (szb + sza) + mz (szb - sza) - c S with
//     S = 2 (sx + sy + szb) and the z factors from per-z tables: one -2c
//     product instead of one per axis, no (pz - mz) / (pz + mz); the
//     conduction coefficient kappa(z) and the DKAPA dT/dz term are folded
//     into the temperature's tables, and the cross-term factors are per-z
//     tables too; with equal x and y spacings (cx1 = cy1) the x and y parts
//     of each advection and induction component share one metric product;
//   * with lShr (no temperature advection or heating) the velocity gradients
//     feed only the induction terms, which are grouped per axis over raw
//     differences with the metric factor applied once per group; without
//     lShr the B differences stay raw and the metric factors ride in u cx1,
//     v cy1, w cz1; OBETA rides in the current density;
//   * the pressure is differenced together with the diagonal momentum flux
//     (P + RU_i u_i, formed once per point, not once per neighbour), and the
//     temperature terms proportional to 1/rho are summed before one multiply;
//   * load_plane forms per point the z differences of u, v, w and the x
//     differences of u, v (difference arrays after the ring), from which the
//     viscous mixed derivatives are one subtraction of two neighbours' values;
//   * repeated gradients are computed once; 1/rho is Newton's iteration
//     r <- r + r(1 - rho r), twice, from the hardware reciprocal estimate.
// Results agree with the reference to rounding (1e-12 of each field's
// max-norm after a step, checked against the oracle).
//
// Wall planes: the values the reference overwrites in BCON (RU, RV, RW, TT,
// BZ and, with lShr, the right-hand side FT) are finite but not the
// reference's before BCON runs; RO, BX, BY and everything on interior planes
// follow the reference.  The z ghost planes are never written (the reference
// only flips RO there between rho and 1/rho; those values reach no result).
#pragma once

#include "mhd_common.cuh"

namespace mhd {
namespace fused {

template <int TX, int TY>
struct Tile {
    static constexpr int kTX = TX;
    static constexpr int kTY = TY;
    static constexpr int kThreads = TX * TY;
    static constexpr int kPX = TX + 2;
    static constexpr int kPY = TY + 2;
    static constexpr int kPlane = kPX * kPY;
};

// quantities held per plane point; Q_PX, Q_PY, Q_PZ are the diagonal momentum
// fluxes P + RU u, P + RV v, P + RW w (P = rho T), which both neighbours of a
// point difference
enum Q { Q_RU = 0, Q_RV, Q_RW, Q_TT, Q_RO, Q_RI, Q_U, Q_V, Q_W, Q_PX, Q_PY, Q_PZ, Q_BX, Q_BY, Q_BZ, Q_N };

template <class SW>
constexpr int nq() {
    return SW::lMag ? Q_N : Q_BX;
}

// per-point differences of the plane being computed, after the ring: the z
// differences of u, v, w and the x differences of u, v (the viscous cross
// terms difference them once more between neighbours)
enum D { D_UZ = 0, D_VZ, D_WZ, D_UX, D_VX, D_N };

template <class SW, class T>
constexpr size_t ring_bytes() {
    return ((size_t)3 * nq<SW>() + D_N) * T::kPlane * sizeof(double);
}

// 1/x by Newton's iteration for the reciprocal, r <- r + r(1 - x r), applied
// twice to the hardware estimate (each step doubles the correct bits).
__device__ __forceinline__ double recip(double x) {
    double r;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
    double e = fma(-x, r, 1.0);
    r = fma(r, e, r);
    e = fma(-x, r, 1.0);
    return fma(r, e, r);
}

// Load plane z into ring slot `slot` with its derived quantities.  With
// `diffs`, also the differences of plane z-1 into the difference arrays: the
// z differences at each point from this plane and plane z-2, which the same
// thread loaded at the same point, and the x differences from plane z-1,
// which a barrier has made visible since its load.
template <class SW, class T>
__device__ __forceinline__ void load_plane(const FusedArgs& a, double* ring, int slot, int z, int x0, int y0,
                                           bool diffs) {
    constexpr int NQ = nq<SW>();
    constexpr int kPlane = T::kPlane, kPX = T::kPX, kThreads = T::kThreads;
    double* base = ring + (size_t)slot * NQ * kPlane;
    const Grid& g = a.g;
    for (int k = threadIdx.x; k < kPlane; k += kThreads) {
        const int hx = k % kPX, hy = k / kPX;
        const int gx = x0 - 1 + hx, gy = y0 - 1 + hy;
        if (gx >= g.nx || gy >= g.ny) continue;
        const long long i = (long long)z * g.sz + (long long)gy * g.sy + gx;
        const double ru = a.U.p[S_RU][i], rv = a.U.p[S_RV][i], rw = a.U.p[S_RW][i];
        const double tt = a.U.p[S_TT][i], ro = a.U.p[S_RO][i];
        const double ri = recip(ro);
        base[Q_RU * kPlane + k] = ru;
        base[Q_RV * kPlane + k] = rv;
        base[Q_RW * kPlane + k] = rw;
        base[Q_TT * kPlane + k] = tt;
        base[Q_RO * kPlane + k] = ro;
        base[Q_RI * kPlane + k] = ri;
        // the stored, rounded products (not contracted into the differences below)
        const double uu = __dmul_rn(ru, ri), vv = __dmul_rn(rv, ri), ww = __dmul_rn(rw, ri);
        base[Q_U * kPlane + k] = uu;
        base[Q_V * kPlane + k] = vv;
        base[Q_W * kPlane + k] = ww;
        const double p = __dmul_rn(ro, tt);
        base[Q_PX * kPlane + k] = fma(ru, uu, p);
        base[Q_PY * kPlane + k] = fma(rv, vv, p);
        base[Q_PZ * kPlane + k] = fma(rw, ww, p);
        if (diffs) {
            const double* Pm2 = ring + (size_t)((slot + 1) % 3) * NQ * kPlane;  // plane z-2
            const double* Pm1 = ring + (size_t)((slot + 2) % 3) * NQ * kPlane;  // plane z-1
            double* Dp = ring + (size_t)3 * NQ * kPlane;
            Dp[D_UZ * kPlane + k] = uu - Pm2[Q_U * kPlane + k];
            Dp[D_VZ * kPlane + k] = vv - Pm2[Q_V * kPlane + k];
            Dp[D_WZ * kPlane + k] = ww - Pm2[Q_W * kPlane + k];
            if (hx >= 1 && hx <= kPX - 2) {
                Dp[D_UX * kPlane + k] = Pm1[Q_U * kPlane + k + 1] - Pm1[Q_U * kPlane + k - 1];
                Dp[D_VX * kPlane + k] = Pm1[Q_V * kPlane + k + 1] - Pm1[Q_V * kPlane + k - 1];
            }
        }
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
    const int yb = (y == 1) ? g.ny - 1 : (y == g.ny - 2 ? 0 : -1);
    const int xb = (x == 1) ? g.nx - 1 : (x == g.nx - 2 ? 0 : -1);
    F[zo + (long long)y * g.sy + x] = v;
    if (xb >= 0) F[zo + (long long)y * g.sy + xb] = v;
    if (yb >= 0) {
        F[zo + (long long)yb * g.sy + x] = v;
        if (xb >= 0) F[zo + (long long)yb * g.sy + xb] = v;
    }
}

// acc + s * D2 F at a node from F[+1], F[-1], F[0], with s folded into
// (c2a_s, c2b_s); HAS_A = false when d2uudu2 vanishes on this axis.
template <bool HAS_A>
__device__ __forceinline__ double acc_d2(double acc, double p, double m, double c, double c2a_s, double c2b_s) {
    acc = fma(fma(-2.0, c, p + m), c2b_s, acc);
    if constexpr (HAS_A) acc = fma(p - m, c2a_s, acc);
    return acc;
}

// One tile (bx, by) of one instance, z planes [zb, ze) of the interior.
// EXTRA: the instantiation with the optional temperature terms (the iTCon 2
// plume heat sink, lRem); the others carry no code for them.  ISO (with UXY):
// cx1 = cy1, the x and y parts of the advection and induction terms summed
// before one metric product.
template <class SW, class T, bool UXY, bool EXTRA = false, bool ISO = false>
__device__ __forceinline__ void substage_tile(const FusedArgs& a, int bx, int by, int zb, int ze, double* ring) {
    constexpr int NQ = nq<SW>();
    constexpr int kTX = T::kTX, kPX = T::kPX, kPlane = T::kPlane, kTY = T::kTY;
    const Grid& g = a.g;
    const Consts& c = a.c;
    const Coefs& K = a.k;
    const int x0 = 1 + bx * kTX, y0 = 1 + by * kTY;
    const int tx = threadIdx.x % kTX, ty = threadIdx.x / kTX;
    const int x = x0 + tx, y = y0 + ty;
    const bool active = (x <= g.nx - 2) && (y <= g.ny - 2);
    const int zl = 1, zr = g.nz - 1;

    // per-column coefficients
    const int xc = active ? x : 1, yc = active ? y : 1;
    const double cx1 = K.cx1[xc], cy1 = K.cy1[yc];
    const double cx2a = K.cx2a[xc], cx2b = K.cx2b[xc], cy2a = K.cy2a[yc], cy2b = K.cy2b[yc];
    // folded viscous / resistive coefficients: [ORE a, ORE b, ORE43 a, ORE43 b, ORM a, ORM b]
    double sx[6], sy[6];
#pragma unroll
    for (int k = 0; k < 6; k++) {
        sx[k] = K.s2[0][k][xc];
        sy[k] = K.s2[1][k][yc];
    }
    const double c13ore = c.C13 * c.ORE;
    const double kxy = c13ore * cx1 * cy1;
    const double kx13 = c13ore * cx1, ky13 = c13ore * cy1;
    // RK coefficients: from the host, or from the device time-step record; a
    // halted record (dt below 1e-8) turns the substage into a copy of U
    const double gdt = a.dtp ? a.gam * a.dtp[0] : a.gdt;
    const double zdt = a.dtp ? a.zet * a.dtp[0] : a.zdt;
    const bool halted = a.dtp && a.dtp[3] != 0.0;
    const double ocvore = c.OCV * c.ORE;
    // the current density carries OBETA (j' = OBETA j): the Lorentz force is
    // B x j' and the Ohmic heating (ORM OCV / OBETA) |j'|^2
    const double ocx1 = c.OBETA * cx1, ocy1 = c.OBETA * cy1;
    const double ohm2 = c.OBETA != 0.0 ? c.ORM * c.OCV / c.OBETA : 0.0;

    load_plane<SW, T>(a, ring, (zb - 1) % 3, zb - 1, x0, y0, false);
    load_plane<SW, T>(a, ring, zb % 3, zb, x0, y0, false);
    __syncthreads();  // plane zb complete: its x differences come with the next load
    load_plane<SW, T>(a, ring, (zb + 1) % 3, zb + 1, x0, y0, true);

    const int pc = (ty + 1) * kPX + (tx + 1);  // centre offset inside a plane
    for (int z = zb; z < ze; z++) {
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
            const double* Dp = ring + (size_t)3 * NQ * kPlane;  // differences of plane z
            auto DD = [&](int d, int off) { return Dp[d * kPlane + pc + off]; };
            const double cz1 = K.cz1[z], cz2a = K.cz2a[z], cz2b = K.cz2b[z];
            double sz[6];
#pragma unroll
            for (int k = 0; k < 6; k++) sz[k] = K.s2[2][k][z];
            auto Dx = [&](int q) { return (XP(q) - XM(q)) * cx1; };
            auto Dy = [&](int q) { return (YP(q) - YM(q)) * cy1; };
            // acc + s * (D2x + D2y + D2z) q with scale pair k (0: ORE, 1: ORE*C43, 2: ORM)
            auto lapx = [&](double acc, int q, int k) { return acc_d2<!UXY>(acc, XP(q), XM(q), C0(q), sx[2 * k], sx[2 * k + 1]); };
            auto lapy = [&](double acc, int q, int k) { return acc_d2<!UXY>(acc, YP(q), YM(q), C0(q), sy[2 * k], sy[2 * k + 1]); };
            auto lapz = [&](double acc, int q, int k) { return acc_d2<true>(acc, ZP(q), ZM(q), C0(q), sz[2 * k], sz[2 * k + 1]); };
            // uniform x / y: acc + sxb (px + mx) + syb (py + my) + pz (szb + sza) + mz (szb - sza) - c S,
            // i.e. the scaled Laplacian with its z part sza (pz - mz) + szb (pz + mz) regrouped;
            // szpm points at the per-z pair of tables (szb + sza, szb - sza), and S = 2 (sxb + syb
            // + szb) comes from a per-z table: one -2c product for the three axes
            auto lap3 = [&](double acc, int q, double sxb, double syb, const double* const* szpm, double S) {
                acc = fma(ZP(q), szpm[0][z], acc);
                acc = fma(ZM(q), szpm[1][z], acc);
                acc = fma(XP(q) + XM(q), sxb, acc);
                acc = fma(YP(q) + YM(q), syb, acc);
                return fma(-C0(q), S, acc);
            };

            const double ro = C0(Q_RO), ri = C0(Q_RI), tt = C0(Q_TT);
            const double u = C0(Q_U), v = C0(Q_V), w = C0(Q_W);
            const long long i = (long long)z * g.sz + (long long)y * g.sy + x;
            // the RK register (read by substages 2 and 3) and FT of this column's
            // next plane into L2, so the next iteration's epilogue does not wait
            // on DRAM for them
            if (z + 1 < ze) {
                const long long inx = i + g.sz;
                if (a.substage != 0) {
#pragma unroll
                    for (int f = 0; f < 8; f++)
                        if (f < (SW::lMag ? 8 : 5)) asm volatile("prefetch.global.L2 [%0];" ::"l"(a.Z.p[f] + inx));
                }
                if constexpr (SW::lShr) asm volatile("prefetch.global.L2 [%0];" ::"l"(a.FT + inx));
            }

            // ---- continuity (3dmhdsub.h:204-227), one-sided dRW/dz on the walls
            double rwz = ZP(Q_RW) - ZM(Q_RW);
            if (z == zl) rwz = 4.0 * ZP(Q_RW) - a.U.p[S_RW][i + 2 * g.sz];
            if (z == zr - 1) rwz = a.U.p[S_RW][i - 2 * g.sz] - 4.0 * ZM(Q_RW);
            const double fr = -fma(rwz, cz1, fma(YP(Q_RV) - YM(Q_RV), cy1, (XP(Q_RU) - XM(Q_RU)) * cx1));

            // ---- pressure, gravity (3dmhdsub.h:266-272) and momentum advection
            // (3dmhdsub.h:279-289): F_i = -D_i P - D_j(RU_i u_j), + GRAV rho in z; the
            // diagonal terms difference P + RU_i u_i, formed once per point by load_plane
            double fu, fv;
            double fw = fma(ro, c.GRAV, -cz1 * (ZP(Q_PZ) - ZM(Q_PZ)));
            if constexpr (ISO) {
                // cx1 = cy1: each component's x and y fluxes are summed before one metric product
                double tu = XP(Q_PX) - XM(Q_PX);
                tu = fma(-YM(Q_RU), YM(Q_V), fma(YP(Q_RU), YP(Q_V), tu));
                double tv = YP(Q_PY) - YM(Q_PY);
                tv = fma(-XM(Q_RV), XM(Q_U), fma(XP(Q_RV), XP(Q_U), tv));
                double tw = fma(XP(Q_RW), XP(Q_U), -XM(Q_RW) * XM(Q_U));
                tw = fma(-YM(Q_RW), YM(Q_V), fma(YP(Q_RW), YP(Q_V), tw));
                fu = -cx1 * tu;
                fv = -cx1 * tv;
                fw = fma(-cx1, tw, fw);
            } else {
                fu = -cx1 * (XP(Q_PX) - XM(Q_PX));
                fv = -cy1 * (YP(Q_PY) - YM(Q_PY));
                fu = fma(-cy1, fma(YP(Q_RU), YP(Q_V), -YM(Q_RU) * YM(Q_V)), fu);
                fv = fma(-cx1, fma(XP(Q_RV), XP(Q_U), -XM(Q_RV) * XM(Q_U)), fv);
                fw = fma(-cx1, fma(XP(Q_RW), XP(Q_U), -XM(Q_RW) * XM(Q_U)), fw);
                fw = fma(-cy1, fma(YP(Q_RW), YP(Q_V), -YM(Q_RW) * YM(Q_V)), fw);
            }
            fu = fma(-cz1, fma(ZP(Q_RU), ZP(Q_W), -ZM(Q_RU) * ZM(Q_W)), fu);
            fv = fma(-cz1, fma(ZP(Q_RV), ZP(Q_W), -ZM(Q_RV) * ZM(Q_W)), fv);

            // ---- temperature: advection (3dmhdsub.h:293-296), conduction (:315-319)
            const double dTz = ZP(Q_TT) - ZM(Q_TT);
            double ft;
            double qr = 0.0;  // the temperature terms proportional to 1/rho, applied once at the end
            // the velocities with their axis' metric factor (the T advection here
            // and the advective induction terms below)
            double cxu = 0.0, cyv = 0.0, czw = 0.0;
            if constexpr (!SW::lShr) {
                cxu = cx1 * u;
                cyv = cy1 * v;
                czw = cz1 * w;
                ft = -fma(cxu, XP(Q_TT) - XM(Q_TT), fma(cyv, YP(Q_TT) - YM(Q_TT), czw * dTz));
            } else {
                ft = a.FT[i];  // the reference never re-initialises FT with lShr
            }
            {
                double lapT = 0.0;
                if constexpr (UXY) {
                    if (EXTRA && c.lrem && !SW::lShr) lapT = lap3(0.0, Q_TT, cx2b, cy2b, K.lapZ + 6, K.lapS[3][z]);
                } else {
                    lapT = acc_d2<true>(0.0, XP(Q_TT), XM(Q_TT), C0(Q_TT), cx2a, cx2b);
                    lapT = acc_d2<true>(lapT, YP(Q_TT), YM(Q_TT), C0(Q_TT), cy2a, cy2b);
                    lapT = acc_d2<true>(lapT, ZP(Q_TT), ZM(Q_TT), C0(Q_TT), cz2a, cz2b);
                }
                if (EXTRA && c.lrem && !SW::lShr) {
                    // lRem: conduction of T - TTM(z) plus HRAD (3dmhdsub.h:297-313),
                    // as lap T + (HRAD - d2 TTM/dz2), the latter precomputed per z
                    ft = fma(ri * (c.OCV / c.REPR), lapT + c.lrem_g[z], ft);
                } else if constexpr (UXY) {
                    // kapz lap T + dkapz dT/dz with kapz folded into per-z coefficients:
                    // condT = kapz (cx2b, cy2b), the pz and mz factors kapz (cz2b + cz2a) + dkapz cz1
                    // and kapz (cz2b - cz2a) - dkapz cz1, and kapz S
                    double q = ZP(Q_TT) * K.condT[2][z];
                    q = fma(ZM(Q_TT), K.condT[3][z], q);
                    q = fma(XP(Q_TT) + XM(Q_TT), K.condT[0][z], q);
                    q = fma(YP(Q_TT) + YM(Q_TT), K.condT[1][z], q);
                    qr = fma(-C0(Q_TT), K.condT[4][z], q);
                } else {
                    ft = fma(ri, fma(K.kapz[z], lapT, K.dkz[z] * dTz), ft);  // dkz = dkapz cz1
                }
            }
            // internal plume heat sink (iTCon 2, 3dmhdsub.h:443-459)
            if constexpr (EXTRA) {
                if (c.pl_mode == 3) qr = fma(-c.pl_s, c.plx[x] * c.ply[y] * c.plz[z], qr);
            }

            // ---- viscous Laplacians (3dmhdsub.h:462-472); scale pairs sx[2k], sx[2k+1]
            if constexpr (UXY) {
                fu = lap3(fu, Q_U, sx[3], sy[1], K.lapZ + 0, K.lapS[0][z]);
                fv = lap3(fv, Q_V, sx[1], sy[3], K.lapZ + 0, K.lapS[1][z]);
                fw = lap3(fw, Q_W, sx[1], sy[1], K.lapZ + 2, K.lapS[2][z]);
            } else {
                fu = lapz(lapy(lapx(fu, Q_U, 1), Q_U, 0), Q_U, 0);
                fv = lapz(lapy(lapx(fv, Q_V, 0), Q_V, 1), Q_V, 0);
                fw = lapz(lapy(lapx(fw, Q_W, 0), Q_W, 0), Q_W, 1);
            }

            // ---- viscous cross terms (3dmhdsub.h:486-487,517-518,531-532)
            {
                double kxz, kyz;
                if constexpr (UXY) {
                    kxz = K.kxz[z];
                    kyz = K.kyz[z];
                } else {
                    kxz = kx13 * cz1;
                    kyz = ky13 * cz1;
                }
                // mixed differences as differences of the neighbours' 1-D differences
                const double dyxv = DD(D_VX, kPX) - DD(D_VX, -kPX);
                const double dyxu = DD(D_UX, kPX) - DD(D_UX, -kPX);
                const double dxzw = DD(D_WZ, 1) - DD(D_WZ, -1);
                const double dyzw = DD(D_WZ, kPX) - DD(D_WZ, -kPX);
                const double dxzu = DD(D_UZ, 1) - DD(D_UZ, -1);
                const double dyzv = DD(D_VZ, kPX) - DD(D_VZ, -kPX);
                fu = fma(kxy, dyxv, fma(kxz, dxzw, fu));
                fv = fma(kxy, dyxu, fma(kyz, dyzw, fv));
                fw = fma(kxz, dxzu, fma(kyz, dyzv, fw));
            }

            // velocity gradients (heating and, without lShr, induction)
            double ux = 0, uy = 0, uz = 0, vx = 0, vy = 0, vz = 0, wx = 0, wy = 0, wz = 0;
            if constexpr (!SW::lShr) {
                ux = DD(D_UX, 0) * cx1; uy = Dy(Q_U); uz = DD(D_UZ, 0) * cz1;
                vx = DD(D_VX, 0) * cx1; vy = Dy(Q_V); vz = DD(D_VZ, 0) * cz1;
                wx = Dx(Q_W); wy = Dy(Q_W); wz = DD(D_WZ, 0) * cz1;
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
                qr = fma(ocvore, phi, qr);
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
                double jx, jy, jz;
                if constexpr (SW::lShr) {
                    // the velocity gradients feed the induction terms only: group each
                    // component's terms by axis over raw differences and apply the axis'
                    // metric factor once per group
                    const double dUx = DD(D_UX, 0), dUy = YP(Q_U) - YM(Q_U), dUz = DD(D_UZ, 0);
                    const double dVx = DD(D_VX, 0), dVy = YP(Q_V) - YM(Q_V), dVz = DD(D_VZ, 0);
                    const double dWx = XP(Q_W) - XM(Q_W), dWy = YP(Q_W) - YM(Q_W);
                    double dWz = DD(D_WZ, 0);
                    // one-sided dw/dz on the walls for the induction terms (3dmhdsub.h:572-584)
                    if (z == zl) {
                        const long long j = i + 2 * g.sz;
                        dWz = 4.0 * ZP(Q_W) - a.U.p[S_RW][j] / a.U.p[S_RO][j];
                    }
                    if (z == zr - 1) {
                        const long long j = i - 2 * g.sz;
                        dWz = a.U.p[S_RW][j] / a.U.p[S_RO][j] - 4.0 * ZM(Q_W);
                    }
                    const double dBXx = XP(Q_BX) - XM(Q_BX), dBXy = YP(Q_BX) - YM(Q_BX), dBXz = ZP(Q_BX) - ZM(Q_BX);
                    const double dBYx = XP(Q_BY) - XM(Q_BY), dBYy = YP(Q_BY) - YM(Q_BY), dBYz = ZP(Q_BY) - ZM(Q_BY);
                    const double dBZx = XP(Q_BZ) - XM(Q_BZ), dBZy = YP(Q_BZ) - YM(Q_BZ), dBZz = ZP(Q_BZ) - ZM(Q_BZ);
                    czw = cz1 * w;
                    if constexpr (ISO) {
                        // cx1 = cy1: each component's x and y terms share one metric product
                        w1 = fma(cx1, fma(-u, dBXx, fma(by, dUy, fma(-v, dBXy, -bx * dVy))),
                                 cz1 * fma(bz, dUz, fma(-w, dBXz, -bx * dWz)));
                        w2 = fma(cx1, fma(-v, dBYy, fma(bx, dVx, fma(-u, dBYx, -by * dUx))),
                                 cz1 * fma(bz, dVz, fma(-w, dBYz, -by * dWz)));
                        w3 = fma(cx1, fma(by, dWy, fma(-v, dBZy, fma(-bz, dVy, fma(bx, dWx, fma(-u, dBZx, -bz * dUx))))),
                                 -czw * dBZz);
                    } else {
                        cxu = cx1 * u;
                        cyv = cy1 * v;
                        w1 = fma(-cxu, dBXx, fma(cy1, fma(by, dUy, fma(-v, dBXy, -bx * dVy)),
                                                 cz1 * fma(bz, dUz, fma(-w, dBXz, -bx * dWz))));
                        w2 = fma(cx1, fma(bx, dVx, fma(-u, dBYx, -by * dUx)),
                                 fma(-cyv, dBYy, cz1 * fma(bz, dVz, fma(-w, dBYz, -by * dWz))));
                        w3 = fma(cx1, fma(bx, dWx, fma(-u, dBZx, -bz * dUx)),
                                 fma(cy1, fma(by, dWy, fma(-v, dBZy, -bz * dVy)), -czw * dBZz));
                    }
                    const double ocz1 = K.ocz1[z];  // OBETA cz1
                    jz = fma(ocx1, dBYx, -ocy1 * dBXy);
                    jy = fma(ocz1, dBXz, -ocx1 * dBZx);
                    jx = fma(ocy1, dBZy, -ocz1 * dBYz);
                } else {
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
                    // raw B differences: the metric factor rides in u cx1, v cy1, w cz1
                    // for the advective terms and in OBETA c for the current density
                    const double dBXx = XP(Q_BX) - XM(Q_BX), dBXy = YP(Q_BX) - YM(Q_BX), dBXz = ZP(Q_BX) - ZM(Q_BX);
                    const double dBYx = XP(Q_BY) - XM(Q_BY), dBYy = YP(Q_BY) - YM(Q_BY), dBYz = ZP(Q_BY) - ZM(Q_BY);
                    const double dBZx = XP(Q_BZ) - XM(Q_BZ), dBZy = YP(Q_BZ) - YM(Q_BZ), dBZz = ZP(Q_BZ) - ZM(Q_BZ);
                    w1 = fma(by, uy, fma(bz, uz, -bx * (vy + wzm)));
                    w1 = fma(-cxu, dBXx, fma(-cyv, dBXy, fma(-czw, dBXz, w1)));
                    w2 = fma(bx, vx, fma(bz, vz, -by * (ux + wzm)));
                    w2 = fma(-cxu, dBYx, fma(-cyv, dBYy, fma(-czw, dBYz, w2)));
                    w3 = fma(bx, wx, fma(by, wy, -bz * (ux + vy)));
                    w3 = fma(-cxu, dBZx, fma(-cyv, dBZy, fma(-czw, dBZz, w3)));
                    const double ocz1 = K.ocz1[z];  // OBETA cz1
                    jz = fma(ocx1, dBYx, -ocy1 * dBXy);
                    jy = fma(ocz1, dBXz, -ocx1 * dBZx);
                    jx = fma(ocy1, dBZy, -ocz1 * dBYz);
                }
                const bool wall = (z == zl || z == zr - 1);
                if constexpr (UXY) {
                    w3 = lap3(w3, Q_BZ, sx[5], sy[5], K.lapZ + 4, K.lapS[4][z]);
                    if (wall) {
                        // x and y parts only: acc + sxb (px + mx) + syb (py + my) - c 2 (sxb + syb)
                        w1 = fma(-bx, K.lapS[5][z], fma(YP(Q_BX) + YM(Q_BX), sy[5], fma(XP(Q_BX) + XM(Q_BX), sx[5], w1)));
                        w2 = fma(-by, K.lapS[5][z], fma(YP(Q_BY) + YM(Q_BY), sy[5], fma(XP(Q_BY) + XM(Q_BY), sx[5], w2)));
                    } else {
                        w1 = lap3(w1, Q_BX, sx[5], sy[5], K.lapZ + 4, K.lapS[4][z]);
                        w2 = lap3(w2, Q_BY, sx[5], sy[5], K.lapZ + 4, K.lapS[4][z]);
                    }
                } else {
                    w1 = lapy(lapx(w1, Q_BX, 2), Q_BX, 2);
                    w2 = lapy(lapx(w2, Q_BY, 2), Q_BY, 2);
                    w3 = lapz(lapy(lapx(w3, Q_BZ, 2), Q_BZ, 2), Q_BZ, 2);
                    if (!wall) {
                        w1 = lapz(w1, Q_BX, 2);
                        w2 = lapz(w2, Q_BY, 2);
                    }
                }
                // d2B/dz2 with the one-sided wall stencils (3dmhdsub.h:640-654,673-687)
                if (wall) {
                    const int s = (z == zl) ? 1 : -1;
                    const long long j2 = i + 2 * s * g.sz, j3 = i + 3 * s * g.sz;
                    const double d2 = c.d2zzdz2[z] * c.hz * c.ORM, d1 = c.dzzdz[z] * c.dzzdz[z] * c.h2z * c.ORM;
                    const double X1 = (s > 0) ? ZP(Q_BX) : ZM(Q_BX), X2 = a.U.p[S_BX][j2], X3 = a.U.p[S_BX][j3];
                    const double Y1 = (s > 0) ? ZP(Q_BY) : ZM(Q_BY), Y2 = a.U.p[S_BY][j2], Y3 = a.U.p[S_BY][j3];
                    const double sg = (double)s;
                    w1 += sg * (-3.0 * bx + 4.0 * X1 - X2) * d2 + (2.0 * bx - 5.0 * X1 + 4.0 * X2 - X3) * d1;
                    w2 += sg * (-3.0 * by + 4.0 * Y1 - Y2) * d2 + (2.0 * by - 5.0 * Y1 + 4.0 * Y2 - Y3) * d1;
                }
                fu = fma(bz, jy, fma(-by, jz, fu));
                fv = fma(bx, jz, fma(-bz, jx, fv));
                fw = fma(by, jx, fma(-bx, jy, fw));
                qr = fma(ohm2, fma(jx, jx, fma(jy, jy, jz * jz)), qr);
            }

            ft = fma(ri, qr, ft);

            // ---- RK3 substage update and the next register (3dmhdsub.h:168-192)
            const double fl[8] = {fu, fv, fw, ft, fr, w1, w2, w3};
            constexpr int nf = SW::lMag ? 8 : 5;
            constexpr int ring_of[8] = {Q_RU, Q_RV, Q_RW, Q_TT, Q_RO, Q_BX, Q_BY, Q_BZ};
#pragma unroll
            for (int f = 0; f < nf; f++) {
                const double zf = (a.substage == 0) ? C0(ring_of[f]) : a.Z.p[f][i];
                const double un = halted ? C0(ring_of[f]) : fma(gdt, fl[f], zf);
                store_with_images(a.Uo.p[f], g, z, y, x, un);
                if (a.substage < 2) a.Z.p[f][i] = halted ? un : fma(zdt, fl[f], un);
            }
            if constexpr (SW::lShr) {
                if (!halted) a.FT[i] = ft;
            }
        }
        __syncthreads();
        if (z + 2 <= ze) load_plane<SW, T>(a, ring, (z + 2) % 3, z + 2, x0, y0, true);
    }
}

// BCON (3dmhdsub.h:720-873) for one wall cell of U' plus its periodic ghost images.
template <class SW>
__device__ __forceinline__ void bcon_cell(const Grid& g, const Consts& c, const Fields8& U, double timt, int wall, int x,
                                          int y) {
    const long long sz = g.sz;
    const double RRT = 1.0, RRB = -1.0, RPP = 0.0;
    const int z = wall == 0 ? 1 : g.nz - 2;
    const int s = wall == 0 ? 1 : -1;
    const long long i = (long long)z * sz + (long long)y * g.sy + x;
    const long long i1 = i + s * sz, i2 = i + 2 * s * sz;
    const double *RU = U.p[S_RU], *RV = U.p[S_RV], *TT = U.p[S_TT], *RO = U.p[S_RO];
    double ru, rv, tt;
    if constexpr (SW::lShr) {
        ru = 0.0;
        rv = (wall == 0 ? RRT : RRB) * cos(RPP * timt) * RO[i];
    } else {
        ru = RO[i] * (c.C43 * RU[i1] / RO[i1] - c.C13 * RU[i2] / RO[i2]);
        rv = RO[i] * (c.C43 * RV[i1] / RO[i1] - c.C13 * RV[i2] / RO[i2]);
    }
    if (wall == 0) {
        if (c.pl_mode == 1) {
            // cooling spot on the top wall (3dmhdsub.h:750-766)
            tt = 1.0f - (1.0f - c.pl_tpr) * c.plx[x] / c.pl_hh * c.ply[y] / c.pl_hh;
        } else if (c.pl_mode == 2) {
            const double DZ = 1.0f / (double)(g.nPz - 1) / c.dzzdz[z];
            tt = c.C43 * TT[i1] - c.C13 * TT[i2] -
                 c.C23 * DZ * (c.THETA - (c.THETA - c.pl_tpr) * c.plx[x] / c.pl_hh * c.ply[y] / c.pl_hh);
        } else if (c.iTCon == 1) {
            const double DZ = 1.0f / (float)(g.nPz - 1) / c.dzzdz[z];
            tt = c.lrem ? c.C43 * TT[i1] - c.C13 * TT[i2] + c.DZTU : c.C43 * TT[i1] - c.C13 * TT[i2] - c.C23 * DZ * c.THETA;
        } else if (c.lrem) {
            tt = c.TU;
        } else {
            tt = 1.0;
            if (c.iTCon == 4 && x < g.nx / 2) tt = 1.0f - c.TP;
        }
    } else {
        if (c.izCon == 0) {
            tt = c.TB;
        } else if (c.lrem) {
            tt = c.C43 * TT[i1] - c.C13 * TT[i2] + c.DZTB;
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

}  // namespace fused
}  // namespace mhd
