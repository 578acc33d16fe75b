"""The split phase of the FP32-sum kernel, restated step for step in numpy
float32 (CPU): its error against the phase in extended precision stays within
the term its error bound carries, 2.5 2^-34 |dt| / P cycles, plus a constant
covered by the column constant err_c0.

The steps follow the device code: the host's 12-bit split of dt = t - t_ref
(joker_abi.cu, prep_star), the float pairs of 1/P and M0 / 2 pi
(joker_math.cuh, prepare_sample and split_d2ff), ih = 1/P with its low 12
mantissa bits cleared (joker_mixed.cuh, mix_consts), then
unit_rv_column_split's phase (joker_fast.cuh).  FMAs are evaluated exactly
in extended precision and rounded once to float32."""
import numpy as np

F32 = np.float32
LD = np.longdouble


def _fma(a, b, c):
    return (LD(1) * a.astype(LD) * b.astype(LD) + c.astype(LD)).astype(F32)


def _split_d2ff(x):
    """hi = x with its mantissa truncated to 24 bits, lo = the rest rounded."""
    b = x.view(np.int64) & ~np.int64((1 << 29) - 1)
    hi = b.view(np.float64).astype(F32)                  # exact: 24 significant bits
    lo = (x - hi.astype(np.float64)).astype(F32)
    return hi, lo


def _prepare(P, M0):
    ph, pl = _split_d2ff(P)
    r0 = F32(1.0) / ph
    t = _fma(-ph, r0, np.ones_like(r0))
    t = _fma(-pl, r0, t)
    r1 = r0 * t
    iph = r0 + r1
    ipl = (r0 - iph) + r1
    mh, ml = _split_d2ff(M0)
    ch = F32(float.fromhex("0x1.45f306p-3"))              # 1 / 2 pi as a float pair
    cl = F32(float.fromhex("0x1.b93910p-28"))
    c = mh * ch
    pe = _fma(mh, np.full_like(mh, ch), -c)
    pe = _fma(mh, np.full_like(mh, cl), pe)
    ce = _fma(ml, np.full_like(ml, ch), pe)
    c = c - np.floor(c)
    mch = c + ce                                          # two-sum
    bb = mch - c
    mcl = (c - (mch - bb)) + (ce - bb)
    return iph, ipl, mch, mcl


def _split_dt(dt):
    mant, ex = np.frexp(dt)
    dth = np.ldexp(np.rint(np.ldexp(mant, 12)), ex - 12)
    return dth.astype(F32), (dt - dth).astype(F32)


def _rint(v, shift):
    if not shift:
        return np.rint(v)
    sh = np.copysign(F32(12582912.0), v).astype(F32)
    return (v + sh) - sh


def _phase(dt, iph, ipl, mch, mcl, shift):
    ih = (iph.view(np.int32) & np.int32(-4096)).view(F32)
    il = (iph - ih) + ipl
    dth, dtl = _split_dt(dt)
    p = dth * ih
    fr = p - _rint(p, shift)
    sm = _fma(dth, il, dtl * iph)
    f0 = (fr - mch) + (sm - mcl)
    return f0 - _rint(f0, shift)


def test_split_phase_error_within_its_bound():
    rng = np.random.default_rng(2024)
    n = 200_000
    P = np.exp(rng.uniform(np.log(0.3), np.log(3000.0), n))
    M0 = rng.uniform(0.0, 2 * np.pi, n)
    dt = rng.uniform(-30000.0, 30000.0, n)
    dt[: n // 10] = rng.uniform(-10.0, 10.0, n // 10)      # short spans: the constant part
    iph, ipl, mch, mcl = _prepare(P, M0)
    exact = dt.astype(LD) / P.astype(LD) - M0.astype(LD) / (LD(2) * LD(np.pi))
    cyc = np.abs(dt) / P
    bound = 2.5 * 2.0 ** -34 * cyc + 2.0 ** -22
    for shift in (False, True):
        f = _phase(dt, iph, ipl, mch, mcl, shift)
        d = (f.astype(LD) - exact).astype(np.float64)
        d -= np.rint(d)                                    # modulo one cycle
        assert np.all(np.abs(d) <= bound), np.max(np.abs(d) / bound)
        # where the proportional term dominates (measured: about 1.3)
        big = cyc > 1e4
        ratio = float(np.max(np.abs(d[big]) / (2.0 ** -34 * cyc[big])))
        print("shift", shift, "largest |error| / (2^-34 |dt|/P) above 1e4 cycles", ratio)
        assert ratio <= 2.5
    # both roundings agree below 2^22 cycles
    assert np.array_equal(_phase(dt, iph, ipl, mch, mcl, False),
                          _phase(dt, iph, ipl, mch, mcl, True))
