"""The certified error bound of the CFL filter's FP32 estimates (CPU).

k_cfl_rows (csrc/mhd_parity.cu) evaluates a cell exactly only when its FP32
estimate of UMACH^2 (as UU/T) or of the fast-mode candidate a0 = DD/sqrt(UU')
lies within 2^-16 of the best estimate seen; DT and UMACH stay bit-exact
because every certified estimate is within 1.4e-6 of the exact FP64 value
(3dmhdsub.h:36-106 computes the exact ones).  This test restates the
estimate in numpy float32 -- IEEE single-precision operations, correctly
rounded like __fadd_rn, __fmul_rn, __frcp_rn, __fsqrt_rn and __fdiv_rn --
with rsqrtf at both ends of its documented 2-ulp error, for both input forms:

* FP64 state: ro, T, momenta and fields truncated to 23 bits (trunc_to_f32);
* FP32 storage: stored floats, ro and T formed as float(rho0) + drho and
  float(T0) + dT in FP32, certified only while |float(profile)| <= 4 |sum|;

and checks the bound on adversarial random inputs across the certified ranges
(ro, T in [2^-20, 2^20], GAMMA in [2^-10, 2^10], OBETA in [0, 2^30]).  For
UMACH^2 the bound is checked where the exact value is at least 2^-41: below
the kernel's 2^-40 threshold no cell is filtered out by it.
"""
import numpy as np
import pytest

f32 = np.float32
BOUND = 1.4e-6
TAU = 2.0 ** -16


def trunc_to_f32(d):
    """Float with d's significand truncated to 23 bits; |d| < 2^-126 -> 0,
    beyond the float range -> inf (the kernel's trunc_to_f32)."""
    b = np.ascontiguousarray(d, dtype=np.float64).view(np.uint64)
    hi = (b >> np.uint64(32)).astype(np.uint32)
    lo = (b & np.uint64(0xffffffff)).astype(np.uint32)
    sign = hi & np.uint32(0x80000000)
    e = ((hi >> np.uint32(20)) & np.uint32(0x7ff)).astype(np.int64) - (1023 - 127)
    mant = ((hi & np.uint32(0x000fffff)) << np.uint32(3)) | (lo >> np.uint32(29))
    out = sign | (np.clip(e, 0, 255).astype(np.uint32) << np.uint32(23)) | mant
    out = np.where(e <= 0, sign, out)
    out = np.where(e >= 255, sign | np.uint32(0x7f800000), out)
    return out.astype(np.uint32).view(np.float32)


def rsqrt_ends(x):
    """rsqrtf(x) at -2 and +2 ulp of the correctly rounded 1/sqrt(x)."""
    r = (1.0 / np.sqrt(x.astype(np.float64))).astype(np.float32)
    lo = np.nextafter(np.nextafter(r, f32(0)), f32(0))
    hi = np.nextafter(np.nextafter(r, f32(np.inf)), f32(np.inf))
    return lo, hi


def estimate(ru, rv, rw, bx, by, bz, ro, tt, okin, ddf, gam_f, obeta_f, mag):
    """cfl_estimate: (a0 at both rsqrtf ends, mc, ok), all float32."""
    with np.errstate(all="ignore"):
        ir = f32(1.0) / ro
        sq = (ru * ru + rv * rv) + rw * rw
        uuk = (sq * ir) * ir
        G = gam_f * tt
        if mag:
            b2 = (bx * bx + by * by) + bz * bz
            G = G + (obeta_f * b2) * ir
        uuf = (uuk + G) + f32(2.0) * np.sqrt(uuk * G)
        mc = uuk / tt
        rlo, rhi = rsqrt_ends(uuf)
        a0s = (ddf * rlo, ddf * rhi)
        ok = (okin & (ro >= f32(2.0 ** -20)) & (ro <= f32(2.0 ** 20)) & (tt >= f32(2.0 ** -20))
              & (tt <= f32(2.0 ** 20)) & np.isfinite(uuf) & np.isfinite(mc)
              & np.isfinite(a0s[0]) & np.isfinite(a0s[1]))
    return a0s, mc, ok


def exact(ru, rv, rw, bx, by, bz, ro, tt, DD, GAMMA, OBETA, mag):
    """The reference's FP64 expressions: UU/T and DD/sqrt(UU')."""
    with np.errstate(all="ignore"):
        UU = (ru * ru + rv * rv + rw * rw) / (ro * ro)
        if mag:
            W = GAMMA * tt + (bx * bx + by * by + bz * bz) * OBETA / ro
            UUp = UU + W + 2.0 * np.sqrt(UU * W)
        else:
            UUp = UU + GAMMA * tt + 2.0 * np.sqrt(GAMMA * UU * tt)
        return UU / tt, DD / np.sqrt(UUp)


def log_uniform(rng, lo, hi, n):
    return np.exp2(rng.uniform(np.log2(lo), np.log2(hi), n))


def signed(rng, lo, hi, n, zero_frac=0.05):
    v = log_uniform(rng, lo, hi, n) * rng.choice([-1.0, 1.0], n)
    v[rng.random(n) < zero_frac] = 0.0
    return v


def _draw(rng, n):
    GAMMA = float(log_uniform(rng, 2.0 ** -10, 2.0 ** 10, 1)[0])
    OBETA = 0.0 if rng.random() < 0.2 else float(log_uniform(rng, 1e-6, 2.0 ** 30, 1)[0])
    DD = float(log_uniform(rng, 1e-4, 1.0, 1)[0])
    ro = log_uniform(rng, 2.0 ** -20, 2.0 ** 20, n)
    tt = log_uniform(rng, 2.0 ** -20, 2.0 ** 20, n)
    scale = np.sqrt(ro * tt)          # momenta around the sound speed times density
    mom = [scale * signed(rng, 1e-12, 1e3, n) for _ in range(3)]
    fld = [np.sqrt(ro * tt) * signed(rng, 1e-12, 1e3, n) for _ in range(3)]
    return GAMMA, OBETA, DD, ro, tt, mom, fld


def _check(a0s, mc, ok, mc_x, a0_x, min_certified=0.8):
    assert ok.sum() > min_certified * ok.size, "too few certified samples to test the bound"
    for a0 in a0s:
        err = np.abs(a0[ok].astype(np.float64) / a0_x[ok] - 1.0)
        assert err.max() <= BOUND, err.max()
    sel = ok & (mc_x >= 2.0 ** -41)
    err = np.abs(mc[sel].astype(np.float64) / mc_x[sel] - 1.0)
    assert err.max() <= BOUND, err.max()
    # the filter margin covers two estimates' errors and the threshold's rounding
    assert TAU > 2 * BOUND + 2.0 ** -23


@pytest.mark.parametrize("mag", [True, False])
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_fp64_state_estimate_bound(mag, seed):
    rng = np.random.default_rng(seed)
    n = 200_000
    GAMMA, OBETA, DD, ro, tt, mom, fld = _draw(rng, n)
    t = [trunc_to_f32(v) for v in mom + fld]
    a0s, mc, ok = estimate(*t, trunc_to_f32(ro), trunc_to_f32(tt), np.ones(n, bool),
                           f32(DD), f32(GAMMA), f32(OBETA), mag)
    mc_x, a0_x = exact(*mom, *fld, ro, tt, DD, GAMMA, OBETA, mag)
    _check(a0s, mc, ok, mc_x, a0_x)


@pytest.mark.parametrize("mag", [True, False])
@pytest.mark.parametrize("seed", [4, 5, 6])
def test_fp32_storage_estimate_bound(mag, seed):
    """Stored floats; ro, T = float(profile) + deviation in FP32; the exact
    values are the FP64 sums profile + widened deviation (as the kernel's
    exact path forms them), including densities and temperatures far below
    the profile (uncertified by the 4:1 guard) and just around it."""
    rng = np.random.default_rng(seed)
    n = 200_000
    GAMMA, OBETA, DD, ro_t, tt_t, mom, fld = _draw(rng, n)
    # profiles within a factor 6 of the targets: some sums cancel past 4:1
    R = ro_t * log_uniform(rng, 1 / 6, 6, n)
    T = tt_t * log_uniform(rng, 1 / 6, 6, n)
    dro = (ro_t - R).astype(np.float32)
    dtt = (tt_t - T).astype(np.float32)
    ro = R + dro.astype(np.float64)
    tt = T + dtt.astype(np.float64)
    Rf, Tf = R.astype(np.float32), T.astype(np.float32)
    with np.errstate(all="ignore"):
        ro_f, tt_f = Rf + dro, Tf + dtt
        okin = (np.abs(Rf) <= f32(4) * np.abs(ro_f)) & (np.abs(Tf) <= f32(4) * np.abs(tt_f))
    assert 0.05 < (~okin).mean() < 0.6  # both sides of the guard are drawn
    s = [v.astype(np.float32) for v in mom + fld]
    a0s, mc, ok = estimate(*s, ro_f, tt_f, okin, f32(DD), f32(GAMMA), f32(OBETA), mag)
    mc_x, a0_x = exact(*[v.astype(np.float64) for v in s], ro, tt, DD, GAMMA, OBETA, mag)
    # the guard's rejects are evaluated exactly; the bound holds for the rest
    _check(a0s, mc, ok, mc_x, a0_x, min_certified=0.4)


def test_guard_is_needed():
    """Without the 4:1 guard the FP32 sum's error is unbounded: a density
    1e5 times below its profile makes the estimate's density (and so its
    UMACH^2) miss by more than the filter margin."""
    R = 1.0 + 2.0 ** -30               # a profile value with bits below float precision
    ro = 1e-5
    dro = np.float32(ro - R)
    ro64 = R + float(dro)
    ro_f = np.float32(np.float32(R) + dro)
    rel = abs(float(ro_f) / ro64 - 1.0)
    assert rel > TAU / 2
    assert abs(np.float32(R)) > 4 * abs(ro_f)  # and the guard rejects it
