// mhd_fp32.cu -- the fused RK3 substage with FP32 field storage.
//
// Storage: every state field is an FP32 array.  RO and TT are stored as
// deviations from an FP64 reference profile rho0(z), T0(z) (the horizontal
// mean of the uploaded state), so the large hydrostatic part of rho and T
// never passes through FP32; the other six fields have a zero profile.
// Arithmetic:
//   FP64: the reconstruction rho = rho0 + drho, T = T0 + dT and the equation
//         of state p = rho T at every point, kept as its deviation
//         dp = p - rho0 T0 from the plane's profile value; the hydrostatic
//         residual of the profiles, rho0 GRAV - D_z(rho0 T0), per z on the
//         host (its two terms nearly cancel); and the RK3 register
//         Z (U' = Z + gamma dt F, Z' = U' + zeta dt F, 3dmhdsub.h:168-192);
//   FP32: every stencil of fluxes() (3dmhdsub.h:204-695), the pressure
//         gradient and gravity among them as stencils of the deviations
//         (-D_x dp, -D_y dp, drho GRAV - D_z dp, added to the residual): the
//         large parts that cancel in hydrostatic balance never pass through
//         FP32.
// The FP64 register Z also carries the state from one step to the next (the
// last substage writes U' into it, BCON keeps its wall values), so FP32
// rounding enters only through the stencil inputs, never into the state.
// The z-march, the shared-memory ring and the ghost-image stores follow the
// FP64 kernel in mhd_fused.cu.
#include "mhd_common.cuh"
#include "mhd_convert.cuh"

#include <type_traits>

namespace mhd {
namespace {

constexpr int kTX = 32;
constexpr int kTY = 8;
constexpr int kThreads = kTX * kTY;
constexpr int kPX = kTX + 2;
constexpr int kPY = kTY + 2;
constexpr int kPlane = kPX * kPY;

// FP32 quantities per plane point; the pressure is kept in FP64 beside them
// F_DP: the pressure deviation p - rho0 T0 of the point (p = rho T in FP64)
enum QF { F_RU = 0, F_RV, F_RW, F_DT, F_DRO, F_RI, F_U, F_V, F_W, F_DP, F_BX, F_BY, F_BZ, F_NQ };

template <class SW>
constexpr int nqf() {
    return SW::lMag ? F_NQ : F_BX;
}

template <class SW>
constexpr size_t plane_bytes() {
    return (size_t)nqf<SW>() * kPlane * sizeof(float);
}

struct RingPtrs {
    float* f;
};

template <class SW>
__device__ __forceinline__ RingPtrs ring_slot(unsigned char* ring, int slot) {
    return {reinterpret_cast<float*>(ring + (size_t)slot * plane_bytes<SW>())};
}

// Raw FP32 fields of one plane (8 with lMag, else 5), staged in shared
// memory by asynchronous copies while the plane two ahead is computed.
template <class SW>
constexpr int nraw() {
    return SW::lMag ? 8 : 5;
}

template <class SW>
constexpr size_t smem_bytes() {
    return 3 * plane_bytes<SW>() + (size_t)nraw<SW>() * kPlane * sizeof(float);
}

template <class SW>
__device__ __forceinline__ float* raw_stage(unsigned char* ring) {
    return reinterpret_cast<float*>(ring + 3 * plane_bytes<SW>());
}

// rho0 and T0 of a plane as float pairs hi + lo (about 48 significant bits)
struct PlanePair {
    float rh, rl, th, tl;
};
__device__ __forceinline__ PlanePair plane_pair(const Fused32Args& a, int z) {
    const int nz = a.g.nz;
    return {a.zf[8 * nz + z], a.zf[9 * nz + z], a.zf[10 * nz + z], a.zf[11 * nz + z]};
}

// The derived quantities of one plane point from its raw fields (get(f) is
// field f of the point): 1/rho and the velocities, and the equation of state
// as the deviation dp = rho T - rho0 T0 of p from the plane's rho0 T0, which
// the x/y differences of the pressure do not see and whose z differences
// enter through the per-z hydrostatic residual.  No FP64 operation: error-free
// FP32 transformations on the float pairs of rho0 and T0 give rho = rh + drho
// exactly as s + e (two-sum), plus rl; and dp = rho0 dT + drho T0 + drho dT
// with every product's rounding error recovered by fma and the three products
// added by two-sums, so dp keeps about one float rounding where those terms
// cancel (near pressure balance; measured against 80-bit sums: <= 0.6 ulp up
// to a 1e6 cancellation ratio, where forming rho T - rho0 T0 in FP64 lost up to
// 4.9e3 ulp).  The _rn intrinsics keep the compiler from contracting or
// reordering the error-free steps.
template <class SW, class Get>
__device__ __forceinline__ void put_point(RingPtrs r, int k, const PlanePair& pp, Get get) {
    const float ru = get(S_RU), rv = get(S_RV), rw = get(S_RW);
    const float dt = get(S_TT), dro = get(S_RO);
    auto two_sum = [](float a, float b, float& e) {
        const float s = __fadd_rn(a, b), bb = __fsub_rn(s, a);
        e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
        return s;
    };
    float se;
    const float s = two_sum(pp.rh, dro, se);
    const float ri = 1.0f / __fadd_rn(s, __fadd_rn(se, pp.rl));
    const float p1 = __fmul_rn(pp.rh, dt), e1 = fmaf(pp.rh, dt, -p1);
    const float p2 = __fmul_rn(pp.th, dro), e2 = fmaf(pp.th, dro, -p2);
    const float p3 = __fmul_rn(dro, dt), e3 = fmaf(dro, dt, -p3);
    float qe, qe2;
    const float q = two_sum(p1, p2, qe);
    const float q2 = two_sum(q, p3, qe2);
    const float tail = ((qe + qe2) + (e1 + e2)) + (e3 + (pp.rl * dt + pp.tl * dro));
    r.f[F_DP * kPlane + k] = __fadd_rn(q2, tail);
    r.f[F_RU * kPlane + k] = ru;
    r.f[F_RV * kPlane + k] = rv;
    r.f[F_RW * kPlane + k] = rw;
    r.f[F_DT * kPlane + k] = dt;
    r.f[F_DRO * kPlane + k] = dro;
    r.f[F_RI * kPlane + k] = ri;
    r.f[F_U * kPlane + k] = ru * ri;
    r.f[F_V * kPlane + k] = rv * ri;
    r.f[F_W * kPlane + k] = rw * ri;
    if constexpr (SW::lMag) {
        r.f[F_BX * kPlane + k] = get(S_BX);
        r.f[F_BY * kPlane + k] = get(S_BY);
        r.f[F_BZ * kPlane + k] = get(S_BZ);
    }
}

// Plane z into ring slot `slot`, read directly from global memory (the first
// three planes of a z range).
template <class SW>
__device__ __forceinline__ void load_plane32(const Fused32Args& a, unsigned char* ring, int slot, int z, int x0,
                                             int y0) {
    RingPtrs r = ring_slot<SW>(ring, slot);
    const Grid& g = a.g;
    const PlanePair pp = plane_pair(a, z);
    for (int k = threadIdx.x; k < kPlane; k += kThreads) {
        const int hx = k % kPX, hy = k / kPX;
        const int gx = x0 - 1 + hx, gy = y0 - 1 + hy;
        if (gx >= g.nx || gy >= g.ny) continue;
        const long long i = (long long)z * g.sz + (long long)gy * g.sy + gx;
        put_point<SW>(r, k, pp, [&](int f) { return a.U.p[f][i]; });
    }
}

// Start the asynchronous copies (cp.async, 4 bytes each: the rows of an
// unpadded FP32 field are not 16-byte aligned) of plane z's raw fields into
// the staging area.  Every thread copies the points it later derives itself,
// so its own cp.async.wait_all is the only wait the derivation needs.
template <class SW>
__device__ __forceinline__ void stage_plane32(const Fused32Args& a, unsigned char* ring, int z, int x0, int y0) {
    float* raw = raw_stage<SW>(ring);
    const Grid& g = a.g;
    for (int k = threadIdx.x; k < kPlane; k += kThreads) {
        const int gx = x0 - 1 + k % kPX, gy = y0 - 1 + k / kPX;
        if (gx >= g.nx || gy >= g.ny) continue;
        const long long i = (long long)z * g.sz + (long long)gy * g.sy + gx;
#pragma unroll
        for (int f = 0; f < nraw<SW>(); f++) {
            const unsigned dst = (unsigned)__cvta_generic_to_shared(raw + f * kPlane + k);
            asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(dst), "l"(a.U.p[f] + i) : "memory");
        }
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
}

// Wait for this thread's staged copies of plane z and derive its points into
// ring slot `slot`.
template <class SW>
__device__ __forceinline__ void derive_plane32(const Fused32Args& a, unsigned char* ring, int slot, int z, int x0,
                                               int y0) {
    asm volatile("cp.async.wait_all;" ::: "memory");
    const float* raw = raw_stage<SW>(ring);
    RingPtrs r = ring_slot<SW>(ring, slot);
    const Grid& g = a.g;
    const PlanePair pp = plane_pair(a, z);
    for (int k = threadIdx.x; k < kPlane; k += kThreads) {
        const int gx = x0 - 1 + k % kPX, gy = y0 - 1 + k / kPX;
        if (gx >= g.nx || gy >= g.ny) continue;
        put_point<SW>(r, k, pp, [&](int f) { return raw[f * kPlane + k]; });
    }
}

__device__ __forceinline__ void store32_with_images(float* F, const Grid& g, int z, int y, int x, float v) {
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

// One tile (bx, by) of one instance, interior z planes [zb, ze).  EXTRA: the
// instantiation with the iTCon 2 plume heat sink.
template <class SW, bool EXTRA = false>
__device__ __forceinline__ void substage32_tile(const Fused32Args& a, int bx, int by, int zb, int ze,
                                                unsigned char* ring) {
    constexpr int NQ = nqf<SW>();
    const Grid& g = a.g;
    const Consts& c = a.c;
    const int x0 = 1 + bx * kTX, y0 = 1 + by * kTY;
    const int tx = threadIdx.x % kTX, ty = threadIdx.x / kTX;
    const int x = x0 + tx, y = y0 + ty;
    const bool active = (x <= g.nx - 2) && (y <= g.ny - 2);
    const int zl = 1, zr = g.nz - 1;

    const int xc = active ? x : 1, yc = active ? y : 1;
    const double cx1d = a.k.cx1[xc], cy1d = a.k.cy1[yc];
    float cx1 = (float)cx1d, cx2a = (float)a.k.cx2a[xc], cx2b = (float)a.k.cx2b[xc];
    float cy1 = (float)cy1d, cy2a = (float)a.k.cy2a[yc], cy2b = (float)a.k.cy2b[yc];
    float c13ore = (float)(c.C13 * c.ORE);
    float kxy = (float)(c.C13 * c.ORE * cx1d * cy1d);
    float ore = (float)c.ORE, ore43 = (float)(c.ORE * c.C43);
    float ocvore = (float)(c.OCV * c.ORE), ocv = (float)c.OCV;
    float ohm = (float)(c.OBETA * c.ORM * c.OCV);
    float tmpc = (float)(c.OCV / c.REPR);
    float obeta = (float)c.OBETA, orm = (float)c.ORM, c43 = (float)c.C43;
    float omz = (float)c.OMZ, omx = (float)c.OMX, grav = (float)c.GRAV;
    // GB300 runs float<->double conversions on its FP64 pipe; under the 80-register
    // cap the compiler would recompute these converted constants inside the z loop
    // (12 conversions per cell, measured).  Opaque copies stay in registers instead.
    asm volatile("" : "+f"(omz), "+f"(omx), "+f"(cx1), "+f"(cx2a), "+f"(cx2b), "+f"(cy1), "+f"(cy2a), "+f"(cy2b));
    asm volatile("" : "+f"(c13ore), "+f"(kxy), "+f"(ore), "+f"(ore43), "+f"(ocvore), "+f"(ocv), "+f"(ohm), "+f"(tmpc));
    asm volatile("" : "+f"(obeta), "+f"(orm), "+f"(c43), "+f"(grav));
    // RK coefficients: from the host, or from the device time-step record; a
    // halted record (dt below 1e-8) turns the substage into a copy of the state
    const double gdt = a.dtp ? a.gam * a.dtp[0] : a.gdt;
    const double zdt = a.dtp ? a.zet * a.dtp[0] : a.zdt;
    const bool halted = a.dtp && a.dtp[3] != 0.0;

    load_plane32<SW>(a, ring, (zb - 1) % 3, zb - 1, x0, y0);
    load_plane32<SW>(a, ring, zb % 3, zb, x0, y0);
    load_plane32<SW>(a, ring, (zb + 1) % 3, zb + 1, x0, y0);

    const int pc = (ty + 1) * kPX + (tx + 1);
    for (int z = zb; z < ze; z++) {
        __syncthreads();
        // plane z+2's raw fields land in the staging area while plane z computes
        if (z + 2 <= ze) stage_plane32<SW>(a, ring, z + 2, x0, y0);
        if (active) {
            const RingPtrs Rm = ring_slot<SW>(ring, (z - 1) % 3);
            const RingPtrs R0 = ring_slot<SW>(ring, z % 3);
            const RingPtrs Rp = ring_slot<SW>(ring, (z + 1) % 3);
            const float* Pm = Rm.f;
            const float* P0 = R0.f;
            const float* Pp = Rp.f;
            auto C0 = [&](int q) { return P0[q * kPlane + pc]; };
            auto XP = [&](int q) { return P0[q * kPlane + pc + 1]; };
            auto XM = [&](int q) { return P0[q * kPlane + pc - 1]; };
            auto YP = [&](int q) { return P0[q * kPlane + pc + kPX]; };
            auto YM = [&](int q) { return P0[q * kPlane + pc - kPX]; };
            auto ZP = [&](int q) { return Pp[q * kPlane + pc]; };
            auto ZM = [&](int q) { return Pm[q * kPlane + pc]; };
            const int nzz = g.nz;
            const float cz1 = a.zf[z], cz2a = a.zf[nzz + z], cz2b = a.zf[2 * nzz + z];
            auto Dx = [&](int q) { return (XP(q) - XM(q)) * cx1; };
            auto Dy = [&](int q) { return (YP(q) - YM(q)) * cy1; };
            auto Dz = [&](int q) { return (ZP(q) - ZM(q)) * cz1; };
            auto D2x = [&](int q) {
                const float p = XP(q), m = XM(q);
                return fmaf(p - m, cx2a, fmaf(-2.0f, C0(q), p + m) * cx2b);
            };
            auto D2y = [&](int q) {
                const float p = YP(q), m = YM(q);
                return fmaf(p - m, cy2a, fmaf(-2.0f, C0(q), p + m) * cy2b);
            };
            auto D2z = [&](int q) {
                const float p = ZP(q), m = ZM(q);
                return fmaf(p - m, cz2a, fmaf(-2.0f, C0(q), p + m) * cz2b);
            };

            const long long i = (long long)z * g.sz + (long long)y * g.sy + x;
            // bring the next plane's FP64 register (and FT) into L2 while this cell computes
            if (z + 1 < ze) {
                const long long inx = i + g.sz;
                constexpr int nfp = SW::lMag ? 8 : 5;
#pragma unroll
                for (int f = 0; f < nfp; f++) asm volatile("prefetch.global.L2 [%0];" ::"l"(a.Z.p[f] + inx));
                if constexpr (SW::lShr) asm volatile("prefetch.global.L2 [%0];" ::"l"(a.FT + inx));
            }
            const float ri = C0(F_RI), ttf = a.zf[10 * nzz + z] + C0(F_DT);  // float(T0) + dT
            const float u = C0(F_U), v = C0(F_V), w = C0(F_W);

            // ---- pressure gradient and gravity (3dmhdsub.h:266-272).  p = p0(z) + dp
            // with p0 = rho0 T0 constant over the plane: x and y see only dp; in z the
            // large, cancelling part rho0 GRAV - D_z p0 is the hydrostatic residual of
            // the profiles, computed per z in FP64 on the host (zf row 7), and the
            // deviations drho GRAV - D_z dp are stenciled here.
            float fu = -(XP(F_DP) - XM(F_DP)) * cx1;
            float fv = -(YP(F_DP) - YM(F_DP)) * cy1;
            float fw = fmaf(C0(F_DRO), grav, fmaf(-(ZP(F_DP) - ZM(F_DP)), cz1, a.zf[7 * nzz + z]));

            // ---- continuity (3dmhdsub.h:204-227)
            float rwz = Dz(F_RW);
            if (z == zl) rwz = (4.0f * ZP(F_RW) - a.U.p[S_RW][i + 2 * g.sz]) * cz1;
            if (z == zr - 1) rwz = (a.U.p[S_RW][i - 2 * g.sz] - 4.0f * ZM(F_RW)) * cz1;
            const float fr = -(Dx(F_RU) + Dy(F_RV) + rwz);

            // ---- momentum advection
            fu -= fmaf(XP(F_RU), XP(F_U), -XM(F_RU) * XM(F_U)) * cx1;
            fu -= fmaf(YP(F_RU), YP(F_V), -YM(F_RU) * YM(F_V)) * cy1;
            fu -= fmaf(ZP(F_RU), ZP(F_W), -ZM(F_RU) * ZM(F_W)) * cz1;
            fv -= fmaf(XP(F_RV), XP(F_U), -XM(F_RV) * XM(F_U)) * cx1;
            fv -= fmaf(YP(F_RV), YP(F_V), -YM(F_RV) * YM(F_V)) * cy1;
            fv -= fmaf(ZP(F_RV), ZP(F_W), -ZM(F_RV) * ZM(F_W)) * cz1;
            fw -= fmaf(XP(F_RW), XP(F_U), -XM(F_RW) * XM(F_U)) * cx1;
            fw -= fmaf(YP(F_RW), YP(F_V), -YM(F_RW) * YM(F_V)) * cy1;
            fw -= fmaf(ZP(F_RW), ZP(F_W), -ZM(F_RW) * ZM(F_W)) * cz1;

            // ---- temperature (deviation stencils plus the FP64 profile's derivatives)
            const float Tz = a.zf[3 * nzz + z] + Dz(F_DT);
            float ft = 0.f;
            if constexpr (!SW::lShr) ft = -fmaf(u, Dx(F_DT), fmaf(v, Dy(F_DT), w * Tz));
            {
                const float lapT = D2x(F_DT) + D2y(F_DT) + (a.zf[4 * nzz + z] + D2z(F_DT));
                ft = fmaf(ri * tmpc, fmaf(a.zf[5 * nzz + z], lapT, a.zf[6 * nzz + z] * Tz), ft);
            }
            // lRem (3dmhdsub.h:297-313): conduction of T - TTM(z) plus HRAD, as
            // lap T + G(z) with G = HRAD - d2 TTM/dz2 from the FP64 plane means;
            // it replaces the kappa(z) conduction term above
            if constexpr (EXTRA && !SW::lShr) {
                if (c.lrem) {
                    const float lapT = D2x(F_DT) + D2y(F_DT) + (a.zf[4 * nzz + z] + D2z(F_DT));
                    ft = -fmaf(u, Dx(F_DT), fmaf(v, Dy(F_DT), w * Tz));
                    ft = fmaf(ri * tmpc, lapT + (float)c.lrem_g[z], ft);
                }
            }
            // internal plume heat sink (iTCon 2, 3dmhdsub.h:443-459)
            if constexpr (EXTRA) {
                if (c.pl_mode == 3)
                    ft = fmaf(-(float)c.pl_s * ri, (float)(c.plx[x] * c.ply[y] * c.plz[z]), ft);
            }

            // ---- viscous Laplacians and cross terms
            fu = fmaf(ore43, D2x(F_U), fmaf(ore, D2y(F_U) + D2z(F_U), fu));
            fv = fmaf(ore43, D2y(F_V), fmaf(ore, D2x(F_V) + D2z(F_V), fv));
            fw = fmaf(ore43, D2z(F_W), fmaf(ore, D2x(F_W) + D2y(F_W), fw));
            {
                const float kxz = c13ore * cx1 * cz1, kyz = c13ore * cy1 * cz1;
                auto E = [&](const float* Pl, int q, int off) { return Pl[q * kPlane + pc + off]; };
                const float dyxv = (E(P0, F_V, kPX + 1) - E(P0, F_V, kPX - 1)) - (E(P0, F_V, -kPX + 1) - E(P0, F_V, -kPX - 1));
                const float dyxu = (E(P0, F_U, kPX + 1) - E(P0, F_U, kPX - 1)) - (E(P0, F_U, -kPX + 1) - E(P0, F_U, -kPX - 1));
                const float dxzw = (E(Pp, F_W, 1) - E(Pm, F_W, 1)) - (E(Pp, F_W, -1) - E(Pm, F_W, -1));
                const float dyzw = (E(Pp, F_W, kPX) - E(Pm, F_W, kPX)) - (E(Pp, F_W, -kPX) - E(Pm, F_W, -kPX));
                const float dxzu = (E(Pp, F_U, 1) - E(Pm, F_U, 1)) - (E(Pp, F_U, -1) - E(Pm, F_U, -1));
                const float dyzv = (E(Pp, F_V, kPX) - E(Pm, F_V, kPX)) - (E(Pp, F_V, -kPX) - E(Pm, F_V, -kPX));
                fu = fmaf(kxy, dyxv, fmaf(kxz, dxzw, fu));
                fv = fmaf(kxy, dyxu, fmaf(kyz, dyzw, fv));
                fw = fmaf(kxz, dxzu, fmaf(kyz, dyzv, fw));
            }
            float ux = 0, uy = 0, uz = 0, vx = 0, vy = 0, vz = 0, wx = 0, wy = 0, wz = 0;
            if constexpr (!SW::lShr || SW::lMag) {
                ux = Dx(F_U); uy = Dy(F_U); uz = Dz(F_U);
                vx = Dx(F_V); vy = Dy(F_V); vz = Dz(F_V);
                wx = Dx(F_W); wy = Dy(F_W); wz = Dz(F_W);
            }
            if constexpr (!SW::lShr) {
                float dg = ux * ux;
                dg = fmaf(vy, vy, dg);
                dg = fmaf(wz, wz, dg);
                dg = fmaf(-ux, vy, dg);
                dg = fmaf(-ux, wz, dg);
                dg = fmaf(-vy, wz, dg);
                const float s1 = uy + vx, s2 = uz + wx, s3 = vz + wy;
                const float sh = fmaf(s1, s1, fmaf(s2, s2, s3 * s3));
                ft = fmaf(ocvore * ri, fmaf(c43, dg, sh), ft);
                ft = fmaf(-ocv * ttf, ux + vy + wz, ft);
            }
            if constexpr (SW::lRot) {
                fu = fmaf(omz, C0(F_RV), fu);
                fv = fmaf(-omz, C0(F_RU), fv);
                fv = fmaf(omx, C0(F_RW), fv);
                fw = fmaf(-omx, C0(F_RV), fw);
            }
            float w1 = 0, w2 = 0, w3 = 0;
            if constexpr (SW::lMag) {
                const float bx = C0(F_BX), by = C0(F_BY), bz = C0(F_BZ);
                float wzm = wz;
                if (z == zl) {
                    const long long j = i + 2 * g.sz;
                    wzm = (4.0f * ZP(F_W) - a.U.p[S_RW][j] / (float)(a.bgR[z + 2] + (double)a.U.p[S_RO][j])) * cz1;
                }
                if (z == zr - 1) {
                    const long long j = i - 2 * g.sz;
                    wzm = (a.U.p[S_RW][j] / (float)(a.bgR[z - 2] + (double)a.U.p[S_RO][j]) - 4.0f * ZM(F_W)) * cz1;
                }
                const float bxx = Dx(F_BX), bxy = Dy(F_BX), bxz = Dz(F_BX);
                const float byx = Dx(F_BY), byy = Dy(F_BY), byz = Dz(F_BY);
                const float bzx = Dx(F_BZ), bzy = Dy(F_BZ), bzz = Dz(F_BZ);
                float lbx = D2x(F_BX) + D2y(F_BX);
                float lby = D2x(F_BY) + D2y(F_BY);
                const float lbz = D2x(F_BZ) + D2y(F_BZ) + D2z(F_BZ);
                if (z == zl || z == zr - 1) {
                    const int s = (z == zl) ? 1 : -1;
                    const long long j2 = i + 2 * s * g.sz, j3 = i + 3 * s * g.sz;
                    const float d2 = (float)(c.d2zzdz2[z] * c.hz), d1 = (float)(c.dzzdz[z] * c.dzzdz[z] * c.h2z);
                    const float X0 = bx, X1 = (s > 0) ? ZP(F_BX) : ZM(F_BX), X2 = a.U.p[S_BX][j2], X3 = a.U.p[S_BX][j3];
                    const float Y0 = by, Y1 = (s > 0) ? ZP(F_BY) : ZM(F_BY), Y2 = a.U.p[S_BY][j2], Y3 = a.U.p[S_BY][j3];
                    const float sg = (float)s;
                    lbx += sg * (-3.0f * X0 + 4.0f * X1 - X2) * d2 + (2.0f * X0 - 5.0f * X1 + 4.0f * X2 - X3) * d1;
                    lby += sg * (-3.0f * Y0 + 4.0f * Y1 - Y2) * d2 + (2.0f * Y0 - 5.0f * Y1 + 4.0f * Y2 - Y3) * d1;
                } else {
                    lbx += D2z(F_BX);
                    lby += D2z(F_BY);
                }
                w1 = fmaf(by, uy, fmaf(bz, uz, -bx * (vy + wzm)));
                w1 = fmaf(-u, bxx, fmaf(-v, bxy, fmaf(-w, bxz, w1)));
                w1 = fmaf(orm, lbx, w1);
                w2 = fmaf(bx, vx, fmaf(bz, vz, -by * (ux + wzm)));
                w2 = fmaf(-u, byx, fmaf(-v, byy, fmaf(-w, byz, w2)));
                w2 = fmaf(orm, lby, w2);
                w3 = fmaf(bx, wx, fmaf(by, wy, -bz * (ux + vy)));
                w3 = fmaf(-u, bzx, fmaf(-v, bzy, fmaf(-w, bzz, w3)));
                w3 = fmaf(orm, lbz, w3);
                const float jz = byx - bxy, jy = bxz - bzx, jx = bzy - byz;
                fu = fmaf(obeta, fmaf(bz, jy, -by * jz), fu);
                fv = fmaf(obeta, fmaf(bx, jz, -bz * jx), fv);
                fw = fmaf(obeta, fmaf(by, jx, -bx * jy), fw);
                ft = fmaf(ohm * ri, fmaf(jx, jx, fmaf(jy, jy, jz * jz)), ft);
            }

            // ---- FP64 RK3 register (3dmhdsub.h:168-192)
            double ftd = widen_f32(ft);
            if constexpr (SW::lShr) ftd += a.FT[i];
            const double fl[8] = {widen_f32(fu), widen_f32(fv), widen_f32(fw), ftd,
                                  widen_f32(fr), widen_f32(w1), widen_f32(w2), widen_f32(w3)};
            const int nf = SW::lMag ? 8 : 5;
            const double r0z = a.bgR[z], t0z = a.bgT[z];
            // Z carries the full FP64 state across steps (written by substage 3
            // and by BCON), so substage 1 starts from it instead of from the
            // FP32 copy: step_block_ZETA0 without the FP32 rounding.  The last
            // substage (and a halted record) stores U' itself into Z; the split
            // keeps its unused register update off the FP64 pipe.
            auto epilogue = [&](auto next_register) {
                // the register fields are read four at a time before any of the
                // four is written: the stores may alias the loads as far as the
                // compiler knows, so a load after a store would wait for it
#pragma unroll
                for (int f0 = 0; f0 < 8; f0 += 4) {
                    if (f0 >= nf) break;
                    double zv[4];
#pragma unroll
                    for (int j = 0; j < 4; j++)
                        if (f0 + j < nf) zv[j] = a.Z.p[f0 + j][i];
#pragma unroll
                    for (int j = 0; j < 4; j++) {
                        const int f = f0 + j;
                        if (f >= nf) break;
                        const double zf = zv[j];
                        const double un = halted ? zf : fma(gdt, fl[f], zf);
                        const double prof = (f == S_TT) ? t0z : (f == S_RO) ? r0z : 0.0;
                        store32_with_images(a.Uo.p[f], g, z, y, x, narrow_f64(un - prof));
                        a.Z.p[f][i] = next_register ? fma(zdt, fl[f], un) : un;
                    }
                }
            };
            if (a.substage < 2 && !halted) epilogue(std::true_type{});
            else epilogue(std::false_type{});
            if constexpr (SW::lShr) {
                if (!halted) a.FT[i] = ftd;
            }
        }
        __syncthreads();
        if (z + 2 <= ze) derive_plane32<SW>(a, ring, (z + 2) % 3, z + 2, x0, y0);
    }
}

// one instance: grid (x tiles, y tiles, z chunks)
template <class SW, bool EXTRA>
__global__ void __launch_bounds__(kThreads, 3) k_substage32(Fused32Args a) {
    extern __shared__ __align__(16) unsigned char ring[];
    const int nPz = a.g.nz - 2;
    const int zb = 1 + (int)((long long)nPz * blockIdx.z / gridDim.z);
    const int ze = 1 + (int)((long long)nPz * (blockIdx.z + 1) / gridDim.z);
    substage32_tile<SW, EXTRA>(a, blockIdx.x, blockIdx.y, zb, ze, ring);
}

// ragged batch: persistent CTAs take (instance, tile x, tile y, z range) items
// (w = first plane | end plane << 16) from a counter that is zero at launch
template <class SW>
__global__ void __launch_bounds__(kThreads, 3) k_substage32_batch(const Fused32Args* __restrict__ args,
                                                               const int4* __restrict__ items, int nitems,
                                                               int* counter, BatchCtl ctl) {
    extern __shared__ __align__(16) unsigned char ring[];
    __shared__ int s_item;
    for (;;) {
        if (threadIdx.x == 0) s_item = atomicAdd(counter, 1);
        __syncthreads();
        const int t = s_item;
        __syncthreads();
        if (t >= nitems) break;
        const int4 it = items[t];
        // a malformed item, or an instance that has taken its steps (both uniform over the CTA)
        if (!batch_item_ok(ctl, args, it, kTX, kTY, SW::lMag ? 8 : 5) || ctl.left[it.x] <= 0) continue;
        substage32_tile<SW>(args[it.x], it.y, it.z, it.w & 0xffff, it.w >> 16, ring);
        __syncthreads();
    }
}

// BCON (3dmhdsub.h:720-873) on the FP32 wall planes, evaluated in FP64 from
// the reconstructed fields, plus the periodic ghost images.
template <class SW>
__device__ __forceinline__ void bcon32_cell(const Grid& g, const Consts& c, const Fields8f& U, const Fields8& Z,
                                            const double* bgR, const double* bgT, double timt, int wall, int x, int y) {
    const long long sz = g.sz;
    const int z = wall == 0 ? 1 : g.nz - 2;
    const int s = wall == 0 ? 1 : -1;
    const long long i = (long long)z * sz + (long long)y * g.sy + x;
    const long long i1 = i + s * sz, i2 = i + 2 * s * sz;
    const float *RU = U.p[S_RU], *RV = U.p[S_RV], *TT = U.p[S_TT], *RO = U.p[S_RO];
    const double ro = bgR[z] + (double)RO[i];
    const double ro1 = bgR[z + s] + (double)RO[i1], ro2 = bgR[z + 2 * s] + (double)RO[i2];
    const double t1 = bgT[z + s] + (double)TT[i1], t2 = bgT[z + 2 * s] + (double)TT[i2];
    double ru, rv, tt;
    if constexpr (SW::lShr) {
        ru = 0.0;
        rv = (wall == 0 ? 1.0 : -1.0) * cos(0.0 * timt) * ro;
    } else {
        ru = ro * (c.C43 * (double)RU[i1] / ro1 - c.C13 * (double)RU[i2] / ro2);
        rv = ro * (c.C43 * (double)RV[i1] / ro1 - c.C13 * (double)RV[i2] / ro2);
    }
    if (wall == 0) {
        if (c.pl_mode == 1) {
            // cooling spot on the top wall (3dmhdsub.h:750-766)
            tt = 1.0f - (1.0f - c.pl_tpr) * c.plx[x] / c.pl_hh * c.ply[y] / c.pl_hh;
        } else if (c.pl_mode == 2) {
            const double DZ = 1.0f / (double)(g.nPz - 1) / c.dzzdz[z];
            tt = c.C43 * t1 - c.C13 * t2 -
                 c.C23 * DZ * (c.THETA - (c.THETA - c.pl_tpr) * c.plx[x] / c.pl_hh * c.ply[y] / c.pl_hh);
        } else if (c.iTCon == 1) {
            const double DZ = 1.0f / (float)(g.nPz - 1) / c.dzzdz[z];
            tt = c.lrem ? c.C43 * t1 - c.C13 * t2 + c.DZTU : c.C43 * t1 - c.C13 * t2 - c.C23 * DZ * c.THETA;
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
            tt = c.C43 * t1 - c.C13 * t2 + c.DZTB;
        } else {
            const double DZ = 1.0f / (float)(g.nPz - 1) / c.dzzdz[z];
            tt = c.C43 * t1 - c.C13 * t2 - c.C23 * DZ * c.THETA / c.RKAPA[z];
        }
    }
    store32_with_images(U.p[S_RU], g, z, y, x, (float)ru);
    store32_with_images(U.p[S_RV], g, z, y, x, (float)rv);
    store32_with_images(U.p[S_RW], g, z, y, x, 0.0f);
    store32_with_images(U.p[S_TT], g, z, y, x, (float)(tt - bgT[z]));
    // the FP64 register holds the state between steps: keep its wall values in step
    Z.p[S_RU][i] = ru;
    Z.p[S_RV][i] = rv;
    Z.p[S_RW][i] = 0.0;
    Z.p[S_TT][i] = tt;
    if constexpr (SW::lMag) {
        if (c.iBCon == 0) {
            store32_with_images(U.p[S_BZ], g, z, y, x, 0.0f);
            Z.p[S_BZ][i] = 0.0;
        }
    }
}

template <class SW>
__global__ void k_bcon_ghost32(Grid g, Consts c, Fields8f U, Fields8 Z, const double* bgR, const double* bgT,
                               double timt) {
    const int nPx = g.nx - 2, nPy = g.ny - 2;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 2 * nPx * nPy) return;
    const int r = t % (nPx * nPy);
    bcon32_cell<SW>(g, c, U, Z, bgR, bgT, timt, t / (nPx * nPy), 1 + r % nPx, 1 + r / nPx);
}

// BCON for a ragged batch: block b covers 128 wall cells of instance items[b].x from cell items[b].y
template <class SW>
__global__ void k_bcon_ghost32_batch(const Fused32Args* __restrict__ args, const int2* __restrict__ items,
                                     BatchCtl ctl) {
    const int2 it = items[blockIdx.x];
    if (it.x < 0 || it.x >= ctl.n) {
        if (threadIdx.x == 0 && atomicCAS(ctl.err, 0, 1) == 0) ctl.err[1] = it.x;
        return;
    }
    if (ctl.left[it.x] <= 0) return;
    const Fused32Args& a = args[it.x];
    const int nPx = a.g.nx - 2, nPy = a.g.ny - 2;
    const int t = it.y + threadIdx.x;
    if (t >= 2 * nPx * nPy) return;
    const int r = t % (nPx * nPy);
    bcon32_cell<SW>(a.g, a.c, a.Uo, a.Z, a.bgR, a.bgT, a.timt, t / (nPx * nPy), 1 + r % nPx, 1 + r / nPx);
}

// periodic ghost fill of FP32 fields (communicate(), 3dmhdmpi.h:11-143)
__global__ void k_comm32(int nf, Grid g, Fields8f U) {
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

// z chunks per column: minimise (waves needed / waves of work) x (planes
// loaded / planes computed) for the reported occupancy
int chunks32(long long tiles, int slots, int nPz) {
    int best = 1;
    double best_cost = 1e300;
    for (int c = 1; c <= 8 && c <= nPz / 4; c++) {
        const double units = (double)tiles * c;
        const double waves = (double)((long long)((units + slots - 1) / slots));
        const double eff = units / (waves * slots);
        const double cost = (1.0 + 2.0 * c / nPz) / eff;
        if (cost < best_cost - 1e-9) {
            best_cost = cost;
            best = c;
        }
    }
    return best;
}

template <class SW, bool EXTRA>
void launch32_t(const Fused32Args& a, cudaStream_t st, int* rc) {
    const size_t smem = smem_bytes<SW>();
    static int slots = 0;
    if (!slots) {
        cudaFuncSetAttribute(k_substage32<SW, EXTRA>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        int dev = 0, sms = 0, per_sm = 1;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_substage32<SW, EXTRA>, kThreads, smem);
        slots = sms * (per_sm > 0 ? per_sm : 1);
    }
    const int nbx = (a.g.nx - 2 + kTX - 1) / kTX, nby = (a.g.ny - 2 + kTY - 1) / kTY;
    const int chunks = chunks32((long long)nbx * nby, slots, a.g.nz - 2);
    k_substage32<SW, EXTRA><<<dim3(nbx, nby, chunks), kThreads, smem, st>>>(a);
    *rc = (int)cudaGetLastError();
}

template <class SW>
void launch32(const Fused32Args& a, cudaStream_t st, int* rc) {
    if (a.c.pl_mode == 3 || a.c.lrem) launch32_t<SW, true>(a, st, rc);
    else launch32_t<SW, false>(a, st, rc);
}

template <class SW>
void launch_bcon32(const Grid& g, const Consts& c, Fields8f U, Fields8 Z, const double* bgR, const double* bgT,
                   double timt, cudaStream_t st) {
    const int n = 2 * (g.nx - 2) * (g.ny - 2);
    k_bcon_ghost32<SW><<<(n + 127) / 128, 128, 0, st>>>(g, c, U, Z, bgR, bgT, timt);
}

template <class SW>
void batch32_launch(const Fused32Args* args, const int4* items, int nitems, int* counter, BatchCtl ctl, int grid,
                    cudaStream_t st, int* rc) {
    k_substage32_batch<SW><<<grid, kThreads, smem_bytes<SW>(), st>>>(args, items, nitems, counter, ctl);
    *rc = (int)cudaGetLastError();
}

template <class SW>
void batch32_occupancy(int* blocks, int* rc) {
    const size_t smem = smem_bytes<SW>();
    cudaFuncSetAttribute(k_substage32_batch<SW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    *rc = (int)cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, k_substage32_batch<SW>, kThreads, smem);
}

template <class SW>
void batch32_bcon(const Fused32Args* args, const int2* items, BatchCtl ctl, int nblocks, cudaStream_t st) {
    k_bcon_ghost32_batch<SW><<<nblocks, 128, 0, st>>>(args, items, ctl);
}

}  // namespace

int fused32_batch_substage(unsigned sw, const Fused32Args* args, const int4* items, int nitems, int* counter,
                           BatchCtl ctl, int grid, cudaStream_t st) {
    int rc = 0;
    MHD_DISPATCH_SW(sw, batch32_launch, args, items, nitems, counter, ctl, grid, st, &rc);
    return rc;
}

int fused32_batch_occupancy(unsigned sw, int* blocks_per_sm) {
    int rc = 0;
    MHD_DISPATCH_SW(sw, batch32_occupancy, blocks_per_sm, &rc);
    return rc;
}

int fused32_batch_bcon(unsigned sw, const Fused32Args* args, const int2* items, BatchCtl ctl, int nblocks,
                       cudaStream_t st) {
    MHD_DISPATCH_SW(sw, batch32_bcon, args, items, ctl, nblocks, st);
    return (int)cudaGetLastError();
}

int fused32_substage(unsigned sw, const Fused32Args& a, cudaStream_t st) {
    int rc = 0;
    MHD_DISPATCH_SW(sw, launch32, a, st, &rc);
    return rc;
}

int fused32_bcon_ghost(unsigned sw, const Grid& g, const Consts& c, Fields8f U, Fields8 Z, const double* bgR,
                       const double* bgT, double timt, cudaStream_t st) {
    MHD_DISPATCH_SW(sw, launch_bcon32, g, c, U, Z, bgR, bgT, timt, st);
    return (int)cudaGetLastError();
}

namespace {

// plane means of T = T0(z) + dT over the interior (y, x), the deviations summed
// in FP64 by a block reduction per plane
__global__ void k_lrem_ttm32(Grid g, const float* dT, const double* bgT, double* ttm) {
    __shared__ double s[256];
    const int z = blockIdx.x;
    const int n = (g.nx - 2) * (g.ny - 2);
    double w = 0;
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const int y = 1 + k / (g.nx - 2), x = 1 + k % (g.nx - 2);
        w += (double)dT[(long long)z * g.sz + (long long)y * g.sy + x];
    }
    s[threadIdx.x] = w;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h) s[threadIdx.x] += s[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) ttm[z] = bgT[z] + s[0] / (double)n;
}

}  // namespace

int lrem_profiles32(const Grid& g, const Consts& c, const float* dT, const double* bgT, double* buf, cudaStream_t st) {
    k_lrem_ttm32<<<g.nz, 256, 0, st>>>(g, dT, bgT, buf);
    const int e = (int)cudaGetLastError();
    return e ? e : lrem_hrad_from_means(g, c, buf, st);
}

int communicate32(int nf, const Grid& g, Fields8f U, cudaStream_t st) {
    const long long n = (2LL * g.nx + 2LL * (g.ny - 2)) * g.nz;
    long long b = (n + 255) / 256;
    if (b > 152 * 16) b = 152 * 16;
    k_comm32<<<(int)b, 256, 0, st>>>(nf, g, U);
    return (int)cudaGetLastError();
}

namespace {

constexpr int kRedThreads = 256;

__device__ __forceinline__ double rec(const Fields8f& U, const double* bg, int f, long long i, int z) {
    const double v = (double)U.p[f][i];
    return bg ? v + bg[z] : v;
}

// Mass, energy, max |div B| and flags in FP64 from the reconstructed state
// (same definitions as the FP64 diagnostics in mhd_diag.cu).
template <bool MAG>
__global__ void k_diag32(Grid g, Consts c, Fields8f U, const double* bgR, const double* bgT, double* part) {
    const int nPx = g.nx - 2, nPy = g.ny - 2, nPz = g.nz - 2;
    const long long ncell = (long long)nPx * nPy * nPz;
    double mass = 0, energy = 0, divb = 0;
    int flags = 0;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < ncell;
         t += (long long)gridDim.x * blockDim.x) {
        const int x = 1 + (int)(t % nPx);
        const int y = 1 + (int)((t / nPx) % nPy);
        const int z = 1 + (int)(t / ((long long)nPx * nPy));
        const long long i = z * g.sz + y * g.sy + x;
        const double ro = rec(U, bgR, S_RO, i, z), tt = rec(U, bgT, S_TT, i, z);
        const double ru = U.p[S_RU][i], rv = U.p[S_RV][i], rw = U.p[S_RW][i];
        const double dv = c.DDX[x] * c.DDY[y] * c.DDZ[z];
        double e = 0.5 * (ru * ru + rv * rv + rw * rw) / ro + c.CV * ro * tt;
        if (!(ro > 0.0)) flags |= 2;
        if (!(tt > 0.0)) flags |= 4;
        if constexpr (MAG) {
            const double bx = U.p[S_BX][i], by = U.p[S_BY][i], bz = U.p[S_BZ][i];
            e += 0.5 * c.OBETA * (bx * bx + by * by + bz * bz);
            if (z > 1 && z < g.nz - 2) {
                const double d = ((double)U.p[S_BX][i + 1] - (double)U.p[S_BX][i - 1]) * c.dxxdx[x] * c.hx +
                                 ((double)U.p[S_BY][i + g.sy] - (double)U.p[S_BY][i - g.sy]) * c.dyydy[y] * c.hy +
                                 ((double)U.p[S_BZ][i + g.sz] - (double)U.p[S_BZ][i - g.sz]) * c.dzzdz[z] * c.hz;
                divb = fmax(divb, fabs(d));
            }
            if (!isfinite(bx) || !isfinite(by) || !isfinite(bz)) flags |= 1;
        }
        if (!isfinite(ro) || !isfinite(tt) || !isfinite(ru) || !isfinite(rv) || !isfinite(rw)) flags |= 1;
        mass += ro * dv;
        energy += e * dv;
    }
    __shared__ double s[4][kRedThreads];
    s[0][threadIdx.x] = mass;
    s[1][threadIdx.x] = energy;
    s[2][threadIdx.x] = divb;
    s[3][threadIdx.x] = (double)flags;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h) {
            s[0][threadIdx.x] += s[0][threadIdx.x + h];
            s[1][threadIdx.x] += s[1][threadIdx.x + h];
            s[2][threadIdx.x] = fmax(s[2][threadIdx.x], s[2][threadIdx.x + h]);
            s[3][threadIdx.x] = (double)((int)s[3][threadIdx.x] | (int)s[3][threadIdx.x + h]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int k = 0; k < 4; k++) part[(long long)k * gridDim.x + blockIdx.x] = s[k][0];
}

__global__ void k_diag32_finish(const double* part, int nb, double* out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double m = 0, e = 0, d = 0;
    int f = 0;
    for (int b = 0; b < nb; b++) {
        m += part[b];
        e += part[nb + b];
        d = fmax(d, part[2LL * nb + b]);
        f |= (int)part[3LL * nb + b];
    }
    out[0] = m;
    out[1] = e;
    out[2] = d;
    out[3] = (double)f;
}

int red_blocks(const Grid& g, int cap) {
    const long long ncell = (long long)(g.nx - 2) * (g.ny - 2) * (g.nz - 2);
    long long nb = (ncell + kRedThreads - 1) / kRedThreads;
    if (nb > cap) nb = cap;
    return nb < 1 ? 1 : (int)nb;
}

}  // namespace


int diag32(bool mag, const Grid& g, const Consts& c, Fields8f U, const double* bgR, const double* bgT,
           double* partials, int max_blocks, double* out4, cudaStream_t st) {
    const int nb = red_blocks(g, max_blocks);
    if (mag) k_diag32<true><<<nb, kRedThreads, 0, st>>>(g, c, U, bgR, bgT, partials);
    else k_diag32<false><<<nb, kRedThreads, 0, st>>>(g, c, U, bgR, bgT, partials);
    k_diag32_finish<<<1, 32, 0, st>>>(partials, nb, out4);
    return (int)cudaGetLastError();
}

}  // namespace mhd
