"""Device-side objects over the C ABI: star tables, the prior cache, the
acceptance pass, and numpy-PCG64 state handling.  PyTorch supplies device
memory and streams only; all arithmetic runs in libjoker_gb300."""
import ctypes

import numpy as np
import torch

from . import _native as nat

__all__ = ["StarTable", "PriorCache", "accept", "stream_handle", "pcg64_state",
           "pcg64_advance_generator", "MaxKeys"]

_MASK128 = (1 << 128) - 1
_PCG_MULT = 0x2360ED051FC65DA44385DF649FCCF645


def stream_handle(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class StarTable:
    """Device-resident table of one or more stars (``joker_stars``), the
    many-star form of CJokerHelper.__init__ (fast_likelihood.pyx:125-253).

    ``stars`` is a list of dicts with keys t, rv, ivar, t_ref, trend_M (N x
    (L-1)), mu, lam (L), k_prior (4: scaled, sigma_K0, P0, max_K).
    """

    def __init__(self, stars, jitter="reference"):
        if not stars:
            raise ValueError("no stars")
        L = len(stars[0]["mu"])
        off = np.zeros(len(stars) + 1, dtype=np.int64)
        for k, s in enumerate(stars):
            off[k + 1] = off[k] + len(s["t"])
            if len(s["mu"]) != L or len(s["lam"]) != L:
                raise ValueError("all stars must share n_linear")
        cat = lambda key: _f64(np.concatenate([np.asarray(s[key], dtype=np.float64) for s in stars]))
        t, rv, ivar = cat("t"), cat("rv"), cat("ivar")
        t_ref = _f64([s["t_ref"] for s in stars])
        if L > 1:
            trend = _f64(np.concatenate([np.asarray(s["trend_M"], dtype=np.float64).reshape(len(s["t"]), L - 1)
                                         for s in stars]))
        else:
            trend = np.zeros(1)
        mu = _f64(np.stack([s["mu"] for s in stars]))
        lam = _f64(np.stack([s["lam"] for s in stars]))
        kp = _f64(np.stack([s["k_prior"] for s in stars]))
        jm = {"reference": nat.JOKER_JITTER_REFERENCE, "applied": nat.JOKER_JITTER_APPLIED}[jitter]
        torch.cuda.init()
        h = ctypes.c_void_p()
        nat.check(nat.lib().joker_stars_create(
            ctypes.byref(h), len(stars), L, nat.lptr(off), nat.dptr(t), nat.dptr(rv),
            nat.dptr(ivar), nat.dptr(t_ref), nat.dptr(trend), nat.dptr(mu), nat.dptr(lam),
            nat.dptr(kp), jm), "joker_stars_create")
        self._h = h
        self.n_stars = len(stars)
        self.n_linear = L
        self.jitter = jitter
        self.epoch_offsets = off
        self.n_epochs = np.diff(off)

    @classmethod
    def slots(cls, n_slots, max_epochs, n_linear, jitter="reference"):
        """An empty slot table (joker_stars_create_slots), filled by ``set``."""
        self = cls.__new__(cls)
        jm = {"reference": nat.JOKER_JITTER_REFERENCE, "applied": nat.JOKER_JITTER_APPLIED}[jitter]
        torch.cuda.init()
        h = ctypes.c_void_p()
        nat.check(nat.lib().joker_stars_create_slots(ctypes.byref(h), int(n_slots),
                                                     int(max_epochs), int(n_linear), jm),
                  "joker_stars_create_slots")
        self._h = h
        self.n_stars = int(n_slots)
        self.n_linear = int(n_linear)
        self.jitter = jitter
        self.max_epochs = int(max_epochs)
        self.n_epochs = None               # filled slot by slot
        return self

    def set(self, slot, star, stream=None):
        """Fill slot ``slot`` with one star (a dict as the constructor takes)."""
        N = len(star["t"])
        L = self.n_linear
        trend = _f64(np.asarray(star["trend_M"], dtype=np.float64).reshape(N, L - 1)) if L > 1 \
            else np.zeros(1)
        t, rv, ivar = _f64(star["t"]), _f64(star["rv"]), _f64(star["ivar"])
        mu, lam, kp = _f64(star["mu"]), _f64(star["lam"]), _f64(star["k_prior"])
        nat.check(nat.lib().joker_stars_set(self.handle, int(slot), N, nat.dptr(t), nat.dptr(rv),
                                            nat.dptr(ivar), float(star["t_ref"]),
                                            nat.dptr(trend), nat.dptr(mu), nat.dptr(lam),
                                            nat.dptr(kp), stream_handle(stream)),
                  "joker_stars_set")

    @property
    def handle(self):
        if self._h is None:
            raise RuntimeError("StarTable is closed")
        return self._h

    def close(self):
        if getattr(self, "_h", None) is not None:
            nat.lib().joker_stars_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PriorCache:
    """Device-resident prior cache (``joker_cache``): the packed (n, 5) samples
    kept as FP64 columns plus the prepared form of the mixed kernel."""

    def __init__(self, capacity):
        torch.cuda.init()
        h = ctypes.c_void_p()
        nat.check(nat.lib().joker_cache_create(ctypes.byref(h), int(capacity)), "joker_cache_create")
        self._h = h
        self.capacity = int(capacity)
        self.size = 0

    @property
    def handle(self):
        if self._h is None:
            raise RuntimeError("PriorCache is closed")
        return self._h

    def load(self, chunk, row0=0, stream=None):
        """Load rows [row0, row0 + len(chunk)) from a (n, 5) float64 array
        (numpy or a CUDA tensor)."""
        if isinstance(chunk, np.ndarray):
            chunk = torch.from_numpy(_f64(chunk)).pin_memory().to("cuda", non_blocking=True)
        if chunk.dtype != torch.float64 or chunk.dim() != 2 or chunk.shape[1] != 5:
            raise ValueError("chunk must be float64 with shape (n, 5)")
        chunk = chunk.contiguous()
        n = chunk.shape[0]
        nat.check(nat.lib().joker_cache_load(self.handle, ctypes.c_void_p(chunk.data_ptr()), n,
                                             int(row0), stream_handle(stream)), "joker_cache_load")
        self.size = max(self.size, int(row0) + n)
        return self

    @classmethod
    def from_samples(cls, chunk, stream=None):
        c = cls(len(chunk))
        return c.load(chunk, 0, stream)

    def sample_prior(self, prior, n=None, seed=0, row0=0, first_index=0, packed=None,
                     stream=None):
        """Draw ``n`` prior samples on the device into rows [row0, row0 + n)
        (joker_prior_sample).  ``prior``: a JokerPrior with the default
        nonlinear priors (LogUniform P, Beta e, uniform angles, s Fixed or
        LogNormal) or a joker_prior_spec field dict.  ``packed``: optional
        (n, 5) float64 CUDA tensor that also receives the samples."""
        n = self.capacity - row0 if n is None else int(n)
        spec = prior_spec(prior)
        if packed is not None:
            if packed.dtype != torch.float64 or tuple(packed.shape) != (n, 5) or \
                    not packed.is_cuda or not packed.is_contiguous():
                raise ValueError("packed must be a contiguous (n, 5) float64 CUDA tensor")
        nat.check(nat.lib().joker_prior_sample(
            self.handle, int(row0), n, ctypes.byref(spec), ctypes.c_uint64(int(seed)),
            int(first_index), ctypes.c_void_p(packed.data_ptr()) if packed is not None else None,
            stream_handle(stream)), "joker_prior_sample")
        self.size = max(self.size, int(row0) + n)
        return self

    @classmethod
    def view(cls, chunk):
        """A cache over a packed (n, 5) float64 chunk without a copy
        (joker_cache_create_view): a CUDA tensor, or a pinned CPU tensor that
        the device reads through its mapped address.  The view keeps a
        reference to the chunk; loading into it is an error."""
        if not isinstance(chunk, torch.Tensor):
            raise TypeError("a cache view takes a torch tensor (CUDA, or pinned CPU)")
        if chunk.dtype != torch.float64 or chunk.dim() != 2 or chunk.shape[1] != 5 or \
                not chunk.is_contiguous():
            raise ValueError("chunk must be a contiguous float64 tensor of shape (n, 5)")
        if not chunk.is_cuda and not chunk.is_pinned():
            raise ValueError("a CPU chunk must be pinned (tensor.pin_memory())")
        torch.cuda.init()
        self = cls.__new__(cls)
        h = ctypes.c_void_p()
        nat.check(nat.lib().joker_cache_create_view(ctypes.byref(h),
                                                    ctypes.c_void_p(chunk.data_ptr()),
                                                    int(chunk.shape[0])),
                  "joker_cache_create_view")
        self._h = h
        self.capacity = self.size = int(chunk.shape[0])
        self._chunk = chunk
        return self

    @classmethod
    def bind(cls, P, e, omega, M0, s):
        """A cache over five float64 columns without a copy (joker_cache_bind):
        1-D tensors of one length, each CUDA or pinned CPU, in the reference's
        internal units.  The view keeps references to the columns."""
        cols = (P, e, omega, M0, s)
        if not all(isinstance(c, torch.Tensor) for c in cols):
            raise TypeError("joker_cache_bind takes torch tensors (CUDA, or pinned CPU)")
        n = int(P.shape[0]) if P.dim() == 1 else -1
        for c in cols:
            if c.dtype != torch.float64 or c.dim() != 1 or c.shape[0] != n or \
                    not c.is_contiguous():
                raise ValueError("columns must be contiguous 1-D float64 tensors of one length")
            if not c.is_cuda and not c.is_pinned():
                raise ValueError("a CPU column must be pinned (tensor.pin_memory())")
        torch.cuda.init()
        self = cls.__new__(cls)
        h = ctypes.c_void_p()
        nat.check(nat.lib().joker_cache_bind(ctypes.byref(h),
                                             *[ctypes.c_void_p(c.data_ptr()) for c in cols], n),
                  "joker_cache_bind")
        self._h = h
        self.capacity = self.size = n
        self._chunk = cols
        return self

    def close(self):
        if getattr(self, "_h", None) is not None:
            nat.lib().joker_cache_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


PRECISIONS = {"fp64": nat.JOKER_FP64, "mixed": nat.JOKER_MIXED,
              "mixed_accurate": nat.JOKER_MIXED_ACCURATE,
              "mixed_fp64_tail": nat.JOKER_MIXED_FP64_TAIL, "mixed_fast": nat.JOKER_MIXED_FAST}


class MaxKeys:
    """Running maxima of ln L (order-preserving uint64 images) on the device."""

    def __init__(self, n):
        self.t = torch.zeros(int(n), dtype=torch.int64, device="cuda")

    def ptr(self):
        return ctypes.c_void_p(self.t.data_ptr())

    def values(self):
        keys = self.t.cpu().numpy().view(np.uint64)
        return np.array([nat.lib().joker_key_to_double(int(k)) for k in keys])


def lnl(stars, cache, out, precision="fp64", star0=0, n_sel=None, row0=0, count=None,
        max_keys=None, err=None, bound_keys=None, chunk=0, out_offset=0, stream=None):
    """ln L of stars [star0, star0 + n_sel) over cache rows [row0, row0 + count)
    into ``out`` (a float64 CUDA tensor of shape (n_sel, ld)).  Mixed
    precisions can also write a per-sample error bound into ``err`` (float32,
    same shape) and the per-star maxima of lnL +- err into ``bound_keys``
    (a MaxKeys of 2 n_sel entries).  Star k's value for row row0 + j goes to
    out[k, out_offset + j]."""
    n_sel = stars.n_stars - star0 if n_sel is None else n_sel
    count = cache.size - row0 if count is None else count
    if out.dtype != torch.float64 or out.dim() != 2 or out.shape[0] < n_sel or \
            out.shape[1] < out_offset + count:
        raise ValueError("out must be float64 with shape (n_sel, >= out_offset + count)")
    if not out.is_contiguous() or (err is not None and (not err.is_contiguous() or
                                                         err.shape != out.shape)):
        raise ValueError("out (and err) must be contiguous, err shaped like out")
    nat.check(nat.lib().joker_lnl(
        stars.handle, cache.handle, int(star0), int(n_sel), int(row0), int(count),
        PRECISIONS[precision], ctypes.c_void_p(out.data_ptr() + 8 * int(out_offset)), out.shape[1],
        max_keys.ptr() if max_keys is not None else None,
        ctypes.c_void_p(err.data_ptr() + 4 * int(out_offset)) if err is not None else None,
        bound_keys.ptr() if bound_keys is not None else None, 0, int(chunk),
        stream_handle(stream)), "joker_lnl")
    return out


# --------------------------------------------------------------------- PCG64
def pcg64_state(rng):
    """(state, inc) of a numpy Generator backed by PCG64, else None."""
    bg = rng.bit_generator
    st = bg.state
    if st.get("bit_generator") != "PCG64":
        return None
    return int(st["state"]["state"]), int(st["state"]["inc"])


def _pcg_advance(state, inc, delta):
    cm, cp, am, ap = _PCG_MULT, inc, 1, 0
    while delta:
        if delta & 1:
            am = (am * cm) & _MASK128
            ap = (ap * cm + cp) & _MASK128
        cp = ((cm + 1) * cp) & _MASK128
        cm = (cm * cm) & _MASK128
        delta >>= 1
    return (am * state + ap) & _MASK128


def pcg64_advance_generator(rng, n_draws):
    """Move a PCG64 Generator forward exactly as ``rng.uniform(size=n_draws)``
    would, leaving its 32-bit buffer untouched."""
    bg = rng.bit_generator
    st = bg.state
    s, inc = int(st["state"]["state"]), int(st["state"]["inc"])
    st["state"]["state"] = _pcg_advance(s, inc, int(n_draws))
    bg.state = st


def pcg64_fields(state, inc, offset=0):
    """Split a PCG64 state advanced by ``offset`` draws for joker_accept_seg."""
    s = _pcg_advance(state, inc, int(offset)) if offset else state
    return s >> 64, s & ((1 << 64) - 1), inc >> 64, inc & ((1 << 64) - 1)


# ----------------------------------------------------------------- acceptance
def _segments(segments, u_source):
    ns = len(segments)
    arr = (nat.AcceptSeg * ns)()
    total_out = 0
    for i, sg in enumerate(segments):
        a = arr[i]
        a.lnl_off, a.n, a.idx_base = int(sg["lnl_off"]), int(sg["n"]), int(sg.get("idx_base", 0))
        a.out_off, a.max_out = int(sg["out_off"]), int(sg["max_out"])
        a.u_off = int(sg.get("u_off", 0))
        a.max_slot = int(sg.get("max_slot", 0))
        a.star = int(sg.get("star", 0))
        a.row0 = int(sg.get("row0", 0))
        if u_source == "pcg64":
            st, inc, off = sg["pcg"]
            a.pcg_state_hi, a.pcg_state_lo, a.pcg_inc_hi, a.pcg_inc_lo = pcg64_fields(st, inc, off)
        total_out = max(total_out, a.out_off + a.max_out)
    return arr, total_out


def refine_max(stars, cache, lnl_buf, err, bound_keys, segments, exact=None, stream=None):
    """FP64 maxima of the segments (joker_refine_max) into ``exact`` (a
    MaxKeys with one slot per max_slot, zeroed here when not given)."""
    ns = len(segments)
    arr, _ = _segments(segments, "array")
    n_slots = max(int(sg.get("max_slot", 0)) for sg in segments) + 1
    if exact is None:
        exact = MaxKeys(n_slots)
    n_ref = torch.zeros(1, dtype=torch.int64, device=lnl_buf.device)
    wbytes = nat.lib().joker_accept_workspace(arr, ns)
    work = torch.empty(max(int(wbytes), 1), dtype=torch.uint8, device=lnl_buf.device)
    nat.check(nat.lib().joker_refine_max(
        stars.handle, cache.handle, arr, ns, ctypes.c_void_p(lnl_buf.data_ptr()),
        ctypes.c_void_p(err.data_ptr()), bound_keys.ptr(), exact.ptr(),
        ctypes.c_void_p(n_ref.data_ptr()), ctypes.c_void_p(work.data_ptr()), int(wbytes),
        stream_handle(stream)), "joker_refine_max")
    if stream is not None:
        work.record_stream(stream)
    return exact, n_ref


def refine_band(stars, cache, lnl_buf, err, exact, segments, band=None, tol=None, stream=None):
    """Band refinement of mixed ln L values (joker_refine_band): every sample
    whose interval reaches within ``band`` of its slot's FP64 maximum
    (``exact``, a MaxKeys from refine_max or accept_refined) and whose bound
    exceeds ``tol`` is re-evaluated in FP64 in place (its bound set to 0).
    Defaults: JOKER_MIXED_LNL_BAND and JOKER_MIXED_LNL_TOL.  Returns the
    number of re-evaluated samples as a one-element CUDA tensor."""
    band = nat.JOKER_MIXED_LNL_BAND if band is None else float(band)
    tol = nat.JOKER_MIXED_LNL_TOL if tol is None else float(tol)
    ns = len(segments)
    arr, _ = _segments(segments, "array")
    n_ref = torch.zeros(1, dtype=torch.int64, device=lnl_buf.device)
    wbytes = nat.lib().joker_accept_workspace(arr, ns)
    work = torch.empty(max(int(wbytes), 1), dtype=torch.uint8, device=lnl_buf.device)
    nat.check(nat.lib().joker_refine_band(
        stars.handle, cache.handle, arr, ns, ctypes.c_void_p(lnl_buf.data_ptr()),
        ctypes.c_void_p(err.data_ptr()), exact.ptr(), band, tol,
        ctypes.c_void_p(n_ref.data_ptr()), ctypes.c_void_p(work.data_ptr()), int(wbytes),
        stream_handle(stream)), "joker_refine_band")
    if stream is not None:
        work.record_stream(stream)
    return n_ref


def accept_refined(stars, cache, lnl_buf, err, bound_keys, segments, u_source="pcg64", u=None,
                   out_idx=None, out_lnl=None, counts=None, exact=None, stream=None):
    """Acceptance over mixed-precision ln L with its error bounds, exact with
    respect to FP64 (joker_accept_refined).  Each segment also names its
    ``star`` and the cache ``row0`` of its first sample.  Returns (out_idx,
    out_lnl, counts, exact_max_keys, n_refined).  ``exact``: FP64 maxima already
    found (joker_refine_max, possibly combined over ranks); computed here when
    None."""
    ns = len(segments)
    arr, total_out = _segments(segments, u_source)
    n_slots = max(int(sg.get("max_slot", 0)) for sg in segments) + 1
    dev = lnl_buf.device
    if out_idx is None:
        out_idx = torch.empty(max(total_out, 1), dtype=torch.int64, device=dev)
    if counts is None:
        counts = torch.empty(ns, dtype=torch.int64, device=dev)
    max_given = exact is not None
    if exact is None:
        exact = MaxKeys(n_slots)
    n_ref = torch.zeros(1, dtype=torch.int64, device=dev)
    wbytes = nat.lib().joker_accept_workspace(arr, ns)
    work = torch.empty(max(int(wbytes), 1), dtype=torch.uint8, device=dev)
    usrc = nat.JOKER_U_PCG64 if u_source == "pcg64" else nat.JOKER_U_ARRAY
    nat.check(nat.lib().joker_accept_refined(
        stars.handle, cache.handle, arr, ns, ctypes.c_void_p(lnl_buf.data_ptr()),
        ctypes.c_void_p(err.data_ptr()), bound_keys.ptr(), exact.ptr(), n_slots,
        int(max_given), usrc,
        ctypes.c_void_p(u.data_ptr()) if u is not None else None,
        ctypes.c_void_p(out_idx.data_ptr()),
        ctypes.c_void_p(out_lnl.data_ptr()) if out_lnl is not None else None,
        ctypes.c_void_p(counts.data_ptr()), ctypes.c_void_p(n_ref.data_ptr()),
        ctypes.c_void_p(work.data_ptr()), int(wbytes), stream_handle(stream)),
        "joker_accept_refined")
    if stream is not None:
        work.record_stream(stream)
    return out_idx, out_lnl, counts, exact, n_ref


def fused_available(stars, precision):
    """Whether ``precision`` on ``stars`` runs the fused first acceptance pass
    (joker_lnl_fused): "mixed_fast", with at most three linear parameters
    when the jitter is applied."""
    return precision == "mixed_fast" and not (stars.jitter == "applied" and stars.n_linear > 3)


def pcg_table(states):
    """Device table of generator states for joker_lnl_fused: one row
    {state_hi, state_lo, inc_hi, inc_lo} per (state, inc) or (state, inc,
    offset) entry of ``states``, as int64 words."""
    rows = []
    for s in states:
        st, inc = s[0], s[1]
        off = s[2] if len(s) > 2 else 0
        rows.append([w - (1 << 64) if w >= (1 << 63) else w for w in pcg64_fields(st, inc, off)])
    return torch.tensor(rows, dtype=torch.int64).view(-1, 4).cuda()


def cand_words(n_sel, n_samples):
    """(cand_ld, tensor) of candidate bits for joker_lnl_fused: n_sel rows of
    cand_ld 32-bit words, enough for n_samples samples per star."""
    ld = ((int(n_samples) + 31) // 32 + 7) // 8 * 8
    return ld, torch.empty((max(int(n_sel), 1), ld), dtype=torch.int32, device="cuda")


def lnl_fused(stars, cache, out, err, bound_keys, pcg, cand, cand_ld, star0=0, n_sel=None,
              row0=0, count=None, first=0, max_keys=None, chunk=0, out_offset=0,
              early_exit=False, stream=None):
    """ln L at "mixed_fast" with the first acceptance pass fused in
    (joker_lnl_fused): as ``lnl``, plus each sample's candidate bit in
    ``cand`` (from cand_words).  ``pcg``: pcg_table of the n_sel stars' streams;
    row row0 + j is number first + j of each stream.  ``early_exit``: warps
    whose samples the partial sums put out of reach stop early; those samples'
    ``out`` holds an upper bound and ``err`` infinity (the kept rows are the
    same)."""
    n_sel = stars.n_stars - star0 if n_sel is None else n_sel
    count = cache.size - row0 if count is None else count
    if out.dtype != torch.float64 or out.dim() != 2 or out.shape[0] < n_sel or \
            out.shape[1] < out_offset + count or not out.is_contiguous():
        raise ValueError("out must be contiguous float64 with shape (n_sel, >= out_offset + count)")
    if err.shape != out.shape or not err.is_contiguous() or err.dtype != torch.float32:
        raise ValueError("err must be contiguous float32 shaped like out")
    nat.check(nat.lib().joker_lnl_fused(
        stars.handle, cache.handle, int(star0), int(n_sel), int(row0), int(count),
        ctypes.c_void_p(pcg.data_ptr()), int(first),
        ctypes.c_void_p(out.data_ptr() + 8 * int(out_offset)), out.shape[1],
        max_keys.ptr() if max_keys is not None else None,
        ctypes.c_void_p(err.data_ptr() + 4 * int(out_offset)), bound_keys.ptr(),
        ctypes.c_void_p(cand.data_ptr()), int(cand_ld), int(chunk), int(bool(early_exit)),
        stream_handle(stream)), "joker_lnl_fused")
    return out


def accept_fused(stars, cache, lnl_buf, err, bound_keys, cand, cand_ld, segments, out_idx=None,
                 out_lnl=None, counts=None, exact=None, stream=None):
    """Second stage of the fused pass (joker_accept_fused): the FP64 maxima
    among the candidates and their decisions; segment s reads its bits from
    row s of ``cand``.  Returns (out_idx, out_lnl, counts, exact_max_keys,
    n_refined) as accept_refined does."""
    ns = len(segments)
    arr, total_out = _segments(segments, "pcg64")
    n_slots = max(int(sg.get("max_slot", 0)) for sg in segments) + 1
    dev = lnl_buf.device
    if out_idx is None:
        out_idx = torch.empty(max(total_out, 1), dtype=torch.int64, device=dev)
    if counts is None:
        counts = torch.empty(ns, dtype=torch.int64, device=dev)
    if exact is None:
        exact = MaxKeys(n_slots)
    n_ref = torch.zeros(1, dtype=torch.int64, device=dev)
    wbytes = nat.lib().joker_accept_workspace(arr, ns)
    work = torch.empty(max(int(wbytes), 1), dtype=torch.uint8, device=dev)
    nat.check(nat.lib().joker_accept_fused(
        stars.handle, cache.handle, arr, ns, ctypes.c_void_p(lnl_buf.data_ptr()),
        ctypes.c_void_p(err.data_ptr()), bound_keys.ptr(), exact.ptr(), n_slots,
        ctypes.c_void_p(cand.data_ptr()), int(cand_ld), ctypes.c_void_p(out_idx.data_ptr()),
        ctypes.c_void_p(out_lnl.data_ptr()) if out_lnl is not None else None,
        ctypes.c_void_p(counts.data_ptr()), ctypes.c_void_p(n_ref.data_ptr()),
        ctypes.c_void_p(work.data_ptr()), int(wbytes), stream_handle(stream)),
        "joker_accept_fused")
    if stream is not None:
        work.record_stream(stream)
    return out_idx, out_lnl, counts, exact, n_ref


def accept(lnl_buf, max_keys, segments, u_source="pcg64", u=None, out_idx=None, out_lnl=None,
           counts=None, stream=None):
    """Run the acceptance pass (joker_accept) over ``segments``.

    Each segment is a dict with lnl_off, n, idx_base, out_off, max_out,
    max_slot and either u_off (u_source="array") or pcg=(state, inc, offset).
    Returns (out_idx, out_lnl, counts) CUDA tensors.
    """
    ns = len(segments)
    arr, total_out = _segments(segments, u_source)
    dev = lnl_buf.device
    if out_idx is None:
        out_idx = torch.empty(max(total_out, 1), dtype=torch.int64, device=dev)
    if counts is None:
        counts = torch.empty(ns, dtype=torch.int64, device=dev)
    wbytes = nat.lib().joker_accept_workspace(arr, ns)
    work = torch.empty(max(int(wbytes), 1), dtype=torch.uint8, device=dev)
    usrc = nat.JOKER_U_PCG64 if u_source == "pcg64" else nat.JOKER_U_ARRAY
    nat.check(nat.lib().joker_accept(
        arr, ns, ctypes.c_void_p(lnl_buf.data_ptr()), max_keys.ptr(), usrc,
        ctypes.c_void_p(u.data_ptr()) if u is not None else None,
        ctypes.c_void_p(out_idx.data_ptr()),
        ctypes.c_void_p(out_lnl.data_ptr()) if out_lnl is not None else None,
        ctypes.c_void_p(counts.data_ptr()), ctypes.c_void_p(work.data_ptr()), int(wbytes),
        stream_handle(stream)), "joker_accept")
    # torch's allocator reuses freed blocks in stream order, so the workspace
    # may be released now; record a foreign stream so that it waits for it
    if stream is not None:
        work.record_stream(stream)
    return out_idx, out_lnl, counts


# ----------------------------------------------------------- after acceptance
def linear_posterior(table, cache, star, rows=None, k_clip=False, stream=None):
    """Posterior of the linear parameters of cache rows ``rows`` (an int64
    CUDA tensor; all rows when None) of one star (joker_linear_posterior):
    (a (n, L), A (n, L, L), ln L (n)) as CUDA float64 tensors."""
    if rows is None:
        rows = torch.arange(cache.size, dtype=torch.int64, device="cuda")
    rows = rows.to(device="cuda", dtype=torch.int64).contiguous()
    n = rows.numel()
    L = table.n_linear
    a = torch.empty((n, L), dtype=torch.float64, device="cuda")
    A = torch.empty((n, L, L), dtype=torch.float64, device="cuda")
    ll = torch.empty(n, dtype=torch.float64, device="cuda")
    nat.check(nat.lib().joker_linear_posterior(
        table.handle, cache.handle, int(star), ctypes.c_void_p(rows.data_ptr()), n,
        int(bool(k_clip)), ctypes.c_void_p(a.data_ptr()), ctypes.c_void_p(A.data_ptr()),
        ctypes.c_void_p(ll.data_ptr()), stream_handle(stream)), "joker_linear_posterior")
    return a, A, ll


def unmarginalized_lnl(table, star, pars, n_trend, dt_shift=0.0, stream=None):
    """ln of the unmarginalized likelihood of full samples
    (joker_unmarginalized_lnl); ``pars``: (n, 6 + n_trend) float64 rows
    P, e, omega, M0, s, K, v_0.. (numpy or CUDA).  Returns a CUDA tensor."""
    if isinstance(pars, np.ndarray):
        pars = torch.from_numpy(_f64(pars))
    pars = pars.to(device="cuda", dtype=torch.float64).contiguous()
    if pars.dim() != 2 or pars.shape[1] != 6 + int(n_trend):
        raise ValueError("pars must have shape (n, 6 + n_trend)")
    n = pars.shape[0]
    out = torch.empty(n, dtype=torch.float64, device="cuda")
    nat.check(nat.lib().joker_unmarginalized_lnl(
        table.handle, int(star), ctypes.c_void_p(pars.data_ptr()), n, int(n_trend),
        float(dt_shift), ctypes.c_void_p(out.data_ptr()), stream_handle(stream)),
        "joker_unmarginalized_lnl")
    return out


def rv_from_elements(t, elems, t0=0.0, stream=None):
    """Radial velocities of Keplerian orbits (joker_rv_from_elements, the
    device counterpart of twobody's c_rv_from_elements): ``t`` (n_t,) times,
    ``elems`` (n, 5) float64 rows P, K, e, omega, M0 (numpy or CUDA).
    Returns an (n, n_t) CUDA tensor, row i = K_i (cos(omega_i + f) + e_i cos
    omega_i) at M = 2 pi (t - t0) / P_i - M0_i."""
    t = torch.as_tensor(_f64(t) if isinstance(t, np.ndarray) else t)
    t = t.to(device="cuda", dtype=torch.float64).reshape(-1).contiguous()
    el = torch.as_tensor(_f64(elems) if isinstance(elems, np.ndarray) else elems)
    el = el.to(device="cuda", dtype=torch.float64).contiguous()
    if el.dim() != 2 or el.shape[1] != 5:
        raise ValueError("elems must have shape (n, 5): P, K, e, omega, M0")
    n, n_t = el.shape[0], t.shape[0]
    out = torch.empty((n, n_t), dtype=torch.float64, device="cuda")
    nat.check(nat.lib().joker_rv_from_elements(
        ctypes.c_void_p(t.data_ptr()), int(n_t), ctypes.c_void_p(el.data_ptr()), n, float(t0),
        ctypes.c_void_p(out.data_ptr()), stream_handle(stream)), "joker_rv_from_elements")
    return out


def prior_spec(prior):
    """joker_prior_spec of a JokerPrior (or of a dict of its fields)."""
    if isinstance(prior, dict):
        f = dict(prior)
        spec = nat.PriorSpec()
        for k, v in f.items():
            setattr(spec, k, v)
        return spec
    from .prior import Beta, Fixed, LogNormal, LogUniform, UniformAngle
    pars = prior.pars
    P, e, om, M0, s = (pars.get(k) for k in ("P", "e", "omega", "M0", "s"))
    if not (isinstance(P, LogUniform) and isinstance(e, Beta) and
            isinstance(om, UniformAngle) and isinstance(M0, UniformAngle) and
            isinstance(s, (Fixed, LogNormal))):
        raise NotImplementedError("device prior sampling covers the default nonlinear priors: "
                                  "LogUniform P, Beta e, uniform omega and M0, Fixed or "
                                  "LogNormal s")
    spec = nat.PriorSpec()
    spec.P_min, spec.P_max = P.a, P.b
    spec.e_alpha, spec.e_beta = e.alpha, e.beta
    if isinstance(s, Fixed):
        spec.s_kind, spec.s_value = nat.JOKER_S_FIXED, s.value
    else:
        spec.s_kind, spec.s_mu, spec.s_sigma = nat.JOKER_S_LOGNORMAL, s.mu, s.sigma
    return spec
