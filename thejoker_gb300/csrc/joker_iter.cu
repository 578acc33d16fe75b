// Iterative rejection sampling for many stars, one device-resident round at a
// time (the rounds can be captured in a CUDA graph and replayed).
//
// Per star this follows iterative_rejection_inmem
// (thejoker/likelihood_helpers.py:130-229):
//   n_process = growth_factor * n_requested (or init_batch_size)
//   loop (at most maxiter rounds):
//     ln L of the next n_process library samples, appended to the star's
//     prefix; uu = rng.uniform(size=len(prefix)) -- fresh draws for the whole
//     prefix every round; keep exp(lnL - max) > uu;
//     stop when n_good >= n_requested; otherwise
//     n_process = int(safety_factor * n_need / n_good * n_evals), clamped to
//     the library, stop when it is <= 0.
// A round is: plan (work items and acceptance segments from the per-star
// state, the star's uniform stream advanced past the draws of earlier
// rounds), the persistent ln L launch over the items, the acceptance pass
// over every active star's prefix, and the update of the state.  Nothing in a
// round allocates, copies from the host or synchronises.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <vector>
#include "joker_internal.cuh"
#include "joker_math.cuh"

namespace joker {
cudaError_t launch_lnl(int precision, int L, bool jit, const LnlArgs &a, int block,
                       cudaStream_t st);
cudaError_t launch_accept(const AcceptArgs &a, int64_t total_blocks, cudaStream_t st,
                          bool max_given);
void set_last_error(const char *msg);
float mixed_err_c0();
}  // namespace joker

using namespace joker;

namespace {

constexpr int ST_START = 0, ST_NPROC = 1, ST_NEVALS = 2, ST_NGOOD = 3, ST_DONE = 4,
              ST_ROUNDS = 5, ST_UCONS = 6, ST_EVAL = 7, ST_FIELDS = 8;
constexpr int64_t DONE_EMPTY = 4;          // a slot without a request
constexpr int64_t BLOCK_SAMPLES = 8192;   // samples per acceptance CTA block

struct IterParams {
    int n_stars;
    int64_t lib_row0;       // cache row of library sample 0
    int chunk;              // samples per ln L work item
    int max_req;            // output slots per star
    int64_t round_budget;   // samples per round over all stars (0: no limit)
    int64_t *cap;           // per star: library size (its prefix grows to at most this)
    int *n_req;             // per star: samples requested
    int64_t *lnl_off;       // per star: offset of its ln L / error buffer in the pool
    double safety;
    int maxiter;
    int64_t *state;
    const uint64_t *pcg0;   // per star: state_hi, state_lo, inc_hi, inc_lo
    joker_accept_seg *segs;
    int64_t *blk_base;      // n_stars + 1
    int64_t *total_blocks;
    int64_t *item_base;     // n_stars + 1: first work item of each star this round
    int64_t *round_row;     // per star: first library row evaluated this round
    int64_t *round_take;    // per star: samples evaluated this round
    WorkItem *items;
    int *n_items;
    unsigned long long *exact_key;
    const int64_t *counts;
    int *done_count;
};

// Exclusive scan of one int64 per thread over a block of 1024 threads; the
// block total goes to *total.
__device__ __forceinline__ int64_t block_exclusive_scan(int64_t v, int64_t *s_warp,
                                                        int64_t *total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int64_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int64_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[wid] = x;
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
        int64_t w = lane < nw ? s_warp[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int64_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < nw) s_warp[lane] = w;         // inclusive warp prefix
    }
    __syncthreads();
    const int64_t excl = x - v + (wid > 0 ? s_warp[wid - 1] : 0);
    *total = s_warp[(blockDim.x >> 5) - 1];
    __syncthreads();
    return excl;
}

// One CTA of 1024 threads.  Pass 1: per active star the samples evaluated
// this round (the rest of its current batch, at most an equal share of the
// round budget) and, for stars whose batch completes, the acceptance segment;
// items and acceptance blocks are scanned over the stars.  Pass 2: the work
// items, all threads over all items.
__global__ void __launch_bounds__(1024) iter_plan_kernel(IterParams p, int zero_exact) {
    __shared__ int64_t s_warp[32];
    __shared__ int s_active;
    if (threadIdx.x == 0) s_active = 0;
    __syncthreads();
    for (int s = threadIdx.x; s < p.n_stars; s += blockDim.x)
        if (p.state[(int64_t)s * ST_FIELDS + ST_DONE] == 0) atomicAdd(&s_active, 1);
    __syncthreads();
    int64_t share = INT64_MAX;
    if (p.round_budget > 0 && s_active > 0) {
        share = max((int64_t)p.chunk, p.round_budget / s_active);
        share = (share + p.chunk - 1) / p.chunk * p.chunk;
    }
    int64_t carry_i = 0, carry_b = 0;
    for (int base = 0; base < p.n_stars; base += blockDim.x) {
        const int s = base + threadIdx.x;
        int64_t nitem = 0, nblk = 0;
        if (s < p.n_stars) {
            int64_t *st = p.state + (int64_t)s * ST_FIELDS;
            joker_accept_seg &g = p.segs[s];
            if (zero_exact) p.exact_key[s] = 0ull;
            g.n = 0;
            if (st[ST_DONE] == 0) {
                const int64_t start = st[ST_START], np = st[ST_NPROC], ev = st[ST_EVAL];
                const int64_t take = min(np - ev, share);
                nitem = (take + p.chunk - 1) / p.chunk;
                p.round_row[s] = start + ev;
                p.round_take[s] = take;
                st[ST_EVAL] = ev + take;
                st[ST_NEVALS] = start + ev + take;
                if (ev + take == np) {
                    // the batch is complete: accept over the whole prefix
                    const int64_t n_evals = start + np;
                    g.n = n_evals;
                    g.lnl_off = p.lnl_off[s];
                    g.out_off = (int64_t)s * p.max_req;
                    g.max_out = p.n_req[s];
                    // the star's uniforms for this acceptance follow those of
                    // its earlier ones in its generator's stream
                    const u128 s0 = ((u128)p.pcg0[4 * s] << 64) | (u128)p.pcg0[4 * s + 1];
                    const u128 inc = ((u128)p.pcg0[4 * s + 2] << 64) | (u128)p.pcg0[4 * s + 3];
                    const u128 sr = pcg_jump(s0, inc, (uint64_t)st[ST_UCONS]);
                    g.pcg_state_hi = (uint64_t)(sr >> 64);
                    g.pcg_state_lo = (uint64_t)sr;
                    g.pcg_inc_hi = p.pcg0[4 * s + 2];
                    g.pcg_inc_lo = p.pcg0[4 * s + 3];
                    nblk = (n_evals + BLOCK_SAMPLES - 1) / BLOCK_SAMPLES;
                }
            }
        }
        int64_t tot_i, tot_b;
        const int64_t ei = block_exclusive_scan(nitem, s_warp, &tot_i);
        const int64_t eb = block_exclusive_scan(nblk, s_warp, &tot_b);
        if (s < p.n_stars) {
            p.item_base[s] = carry_i + ei;
            p.blk_base[s] = carry_b + eb;
        }
        carry_i += tot_i;
        carry_b += tot_b;
    }
    if (threadIdx.x == 0) {
        p.item_base[p.n_stars] = carry_i;
        p.blk_base[p.n_stars] = carry_b;
        *p.total_blocks = carry_b;
        *p.n_items = (int)carry_i;
    }
    __syncthreads();
    // pass 2: item k belongs to the last star whose first item is <= k
    for (int64_t k = threadIdx.x; k < carry_i; k += blockDim.x) {
        int lo = 0, hi = p.n_stars;          // item_base[lo] <= k < item_base[hi]
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (p.item_base[mid] <= k) lo = mid; else hi = mid;
        }
        const int64_t c = k - p.item_base[lo];
        const int64_t r = p.round_row[lo] + c * p.chunk;
        const int64_t rem = p.round_take[lo] - c * p.chunk;
        WorkItem w;
        w.star = lo;
        w.row0 = p.lib_row0 + r;
        w.count = (int)(rem < p.chunk ? rem : p.chunk);
        w.out_off = p.lnl_off[lo] + r;
        w.max_slot = lo;
        w.pad = 0;
        p.items[k] = w;
    }
}

// One thread per star: the growth rule of likelihood_helpers.py:187-211.
__global__ void iter_update_kernel(IterParams p) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= p.n_stars) return;
    int64_t *st = p.state + (int64_t)s * ST_FIELDS;
    if (st[ST_DONE] != 0) return;
    if (st[ST_EVAL] < st[ST_NPROC]) return;   // the batch continues next round
    st[ST_EVAL] = 0;
    const int64_t n_good = p.counts[s];
    const int64_t n_evals = st[ST_NEVALS];
    st[ST_NGOOD] = n_good;
    st[ST_UCONS] += n_evals;                 // this round drew len(prefix) uniforms
    st[ST_ROUNDS] += 1;
    int64_t done = 0;
    if (n_good == 0) {
        done = 2;                            // "Failed to find any good samples!"
    } else if (n_good >= p.n_req[s]) {
        done = 1;
    } else {
        const int64_t start = st[ST_START] + st[ST_NPROC];
        const int64_t n_need = p.n_req[s] - n_good;
        double v = p.safety * (double)n_need / (double)n_good * (double)n_evals;
        int64_t np = (int64_t)v;
        if (start + np > p.cap[s]) np = p.cap[s] - start;
        st[ST_START] = start;
        st[ST_NPROC] = np;
        if (np <= 0) done = 1;               // the library is exhausted: keep what passed
        else if (st[ST_ROUNDS] >= p.maxiter) done = 3;
    }
    if (done) {
        st[ST_DONE] = done;
        atomicAdd(p.done_count, 1);
    }
}

// Start a request in slot s (between rounds): its schedule, pool buffer and
// uniform stream; the slot's running maxima are reset.
__global__ void iter_admit_kernel(IterParams p, unsigned long long *max_key,
                                  unsigned long long *bound_key, int s, int64_t budget, int n_req,
                                  int64_t init, int64_t pool_off, uint64_t s_hi, uint64_t s_lo,
                                  uint64_t i_hi, uint64_t i_lo) {
    int64_t *st = p.state + (int64_t)s * ST_FIELDS;
    // the finished count covers slots holding a finished request
    if (st[ST_DONE] >= 1 && st[ST_DONE] <= 3) atomicSub(p.done_count, 1);
    for (int f = 0; f < ST_FIELDS; ++f) st[f] = 0;
    st[ST_NPROC] = init;
    p.cap[s] = budget;
    p.n_req[s] = n_req;
    p.lnl_off[s] = pool_off;
    uint64_t *pc = const_cast<uint64_t *>(p.pcg0) + 4 * s;
    pc[0] = s_hi; pc[1] = s_lo; pc[2] = i_hi; pc[3] = i_lo;
    max_key[s] = 0ull;
    bound_key[2 * s] = 0ull;
    bound_key[2 * s + 1] = 0ull;
}

}  // namespace

struct joker_iter {
    const joker_stars *stars = nullptr;
    const joker_cache *cache = nullptr;
    int precision = 0;
    int L = 0, jit = 0;
    IterParams p{};
    int64_t max_blocks = 0, items_cap = 0, pool = 0;
    void *base = nullptr;                    // one allocation holds every buffer
    double *lnl = nullptr;
    float *err = nullptr;
    unsigned long long *max_key = nullptr, *bound_key = nullptr;
    uint32_t *words = nullptr, *amb = nullptr;
    int64_t *blk_count = nullptr, *counts = nullptr, *out_idx = nullptr;
    double *out_lnl = nullptr;
    unsigned long long *n_refined = nullptr;
    int *queue = nullptr;
    unsigned long long *flag_count = nullptr;
    int64_t *flag_list = nullptr;
    int64_t flag_cap = 0;
};

// stars/cache accessors live in joker_abi.cu
namespace joker {
void stars_internals(const joker_stars *s, const StarRec **recs, const double **ep64,
                     const float **ep32, int *n_stars, int *L, int *jit, int **queue);
void cache_internals(const joker_cache *c, int64_t *cap, const double **P, const double **E,
                     const double **OM, const double **M0, const double **S, int64_t *stride,
                     const float4 **mx_a, const float4 **mx_b, const float **mx_s2);
}  // namespace joker

static int iter_fail(int code, const char *msg) {
    set_last_error(msg);
    return code;
}

static size_t al(size_t x) { return (x + 255) & ~(size_t)255; }

// Allocate a handle for n_slots stars whose ln L prefixes share a pool of
// pool_samples samples.  Every slot starts empty.
static int iter_alloc(joker_iter **out, const joker_stars *stars, const joker_cache *cache,
                      int precision, int64_t lib_row0, int64_t pool_samples, int max_req,
                      double safety_factor, int maxiter, int chunk, const char *who) {
    char buf[256];
    if (!out || !stars || !cache) {
        snprintf(buf, sizeof buf, "%s: NULL argument", who);
        return iter_fail(JOKER_EINVAL, buf);
    }
    *out = nullptr;
    const StarRec *recs; const double *ep64; const float *ep32; int n_stars, L, jit; int *queue;
    stars_internals(stars, &recs, &ep64, &ep32, &n_stars, &L, &jit, &queue);
    int64_t cap, cstride; const double *P, *E, *OM, *M0, *S; const float4 *ma, *mb; const float *ms;
    cache_internals(cache, &cap, &P, &E, &OM, &M0, &S, &cstride, &ma, &mb, &ms);
    if (lib_row0 < 0 || lib_row0 >= cap || pool_samples <= 0 || max_req <= 0 || maxiter <= 0 ||
        !(safety_factor > 0)) {
        snprintf(buf, sizeof buf, "%s: bad library, pool or schedule parameters", who);
        return iter_fail(JOKER_EINVAL, buf);
    }
    if (precision != JOKER_FP64 && precision != JOKER_MIXED && precision != JOKER_MIXED_ACCURATE &&
        precision != JOKER_MIXED_FAST) {
        snprintf(buf, sizeof buf, "%s: precision must be FP64 or a mixed precision with error "
                                  "bounds", who);
        return iter_fail(JOKER_EINVAL, buf);
    }
    if (chunk <= 0) chunk = 1024;
    joker_iter *it = new joker_iter();
    it->stars = stars;
    it->cache = cache;
    it->precision = precision;
    it->L = L;
    it->jit = jit;
    const int n = n_stars;
    it->pool = pool_samples;
    it->max_blocks = pool_samples / BLOCK_SAMPLES + n + 1;
    it->items_cap = pool_samples / chunk + n + 1;
    const bool mixed = precision != JOKER_FP64;
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off += al(bytes); return o; };
    const size_t o_state = take(8 * (size_t)n * ST_FIELDS), o_pcg = take(32 * (size_t)n),
                 o_cap = take(8 * (size_t)n), o_nreq = take(4 * (size_t)n),
                 o_loff = take(8 * (size_t)n),
                 o_segs = take(sizeof(joker_accept_seg) * (size_t)n),
                 o_base = take(8 * ((size_t)n + 1)), o_tot = take(8),
                 o_ibase = take(8 * ((size_t)n + 1)), o_rrow = take(8 * (size_t)n),
                 o_rtake = take(8 * (size_t)n),
                 o_items = take(sizeof(WorkItem) * (size_t)it->items_cap), o_nitems = take(4),
                 o_exact = take(8 * (size_t)n), o_done = take(4),
                 o_lnl = take(8 * (size_t)pool_samples),
                 o_err = mixed ? take(4 * (size_t)pool_samples) : 0, o_mk = take(8 * (size_t)n),
                 o_bk = take(16 * (size_t)n), o_words = take(4 * 256 * (size_t)it->max_blocks),
                 o_amb = take(4 * 256 * (size_t)it->max_blocks),
                 o_bc = take(8 * (size_t)it->max_blocks), o_cnt = take(8 * (size_t)n),
                 o_oidx = take(8 * (size_t)n * max_req), o_olnl = take(8 * (size_t)n * max_req),
                 o_nref = take(8), o_queue = take(16),
                 o_fcount = take(16), o_flags = take(8 * (size_t)(65536 + 64 * it->max_blocks));
    cudaError_t e = cudaMalloc(&it->base, off);
    if (e != cudaSuccess) {
        delete it;
        snprintf(buf, sizeof buf, "%s: cudaMalloc(%zu): %s", who, off, cudaGetErrorString(e));
        return iter_fail(JOKER_ENOMEM, buf);
    }
    char *b = (char *)it->base;
    IterParams &p = it->p;
    p.n_stars = n;
    p.lib_row0 = lib_row0;
    p.chunk = chunk;
    p.max_req = max_req;
    p.cap = (int64_t *)(b + o_cap);
    p.n_req = (int *)(b + o_nreq);
    p.lnl_off = (int64_t *)(b + o_loff);
    p.safety = safety_factor;
    p.maxiter = maxiter;
    p.state = (int64_t *)(b + o_state);
    p.pcg0 = (const uint64_t *)(b + o_pcg);
    p.segs = (joker_accept_seg *)(b + o_segs);
    p.blk_base = (int64_t *)(b + o_base);
    p.total_blocks = (int64_t *)(b + o_tot);
    p.item_base = (int64_t *)(b + o_ibase);
    p.round_row = (int64_t *)(b + o_rrow);
    p.round_take = (int64_t *)(b + o_rtake);
    p.round_budget = 0;
    p.items = (WorkItem *)(b + o_items);
    p.n_items = (int *)(b + o_nitems);
    p.exact_key = (unsigned long long *)(b + o_exact);
    p.done_count = (int *)(b + o_done);
    it->lnl = (double *)(b + o_lnl);
    it->err = mixed ? (float *)(b + o_err) : nullptr;
    it->max_key = (unsigned long long *)(b + o_mk);
    it->bound_key = (unsigned long long *)(b + o_bk);
    it->words = (uint32_t *)(b + o_words);
    it->amb = (uint32_t *)(b + o_amb);
    it->blk_count = (int64_t *)(b + o_bc);
    it->counts = (int64_t *)(b + o_cnt);
    p.counts = it->counts;
    it->out_idx = (int64_t *)(b + o_oidx);
    it->out_lnl = (double *)(b + o_olnl);
    it->n_refined = (unsigned long long *)(b + o_nref);
    it->queue = (int *)(b + o_queue);
    it->flag_count = (unsigned long long *)(b + o_fcount);
    it->flag_list = (int64_t *)(b + o_flags);
    it->flag_cap = 65536 + 64 * it->max_blocks;
    // every slot empty; the constant parts of the segments
    std::vector<int64_t> st((size_t)n * ST_FIELDS, 0);
    for (int s = 0; s < n; ++s) st[(size_t)s * ST_FIELDS + ST_DONE] = DONE_EMPTY;
    std::vector<joker_accept_seg> segs(n);
    memset(segs.data(), 0, sizeof(joker_accept_seg) * n);
    for (int s = 0; s < n; ++s) {
        segs[s].max_slot = s;
        segs[s].star = s;
        segs[s].row0 = lib_row0;
    }
    if ((e = cudaMemset(it->base, 0, off)) != cudaSuccess ||
        (e = cudaMemcpy(p.state, st.data(), 8 * st.size(), cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(p.segs, segs.data(), sizeof(joker_accept_seg) * n, cudaMemcpyHostToDevice)) != cudaSuccess) {
        cudaFree(it->base);
        delete it;
        snprintf(buf, sizeof buf, "%s: initialisation failed: %s", who, cudaGetErrorString(e));
        return iter_fail(JOKER_ECUDA, buf);
    }
    *out = it;
    return JOKER_OK;
}

extern "C" int joker_iter_admit(joker_iter *it, int slot, int64_t budget, int n_requested,
                                int64_t init_batch, int64_t pool_off, const uint64_t *pcg_state,
                                void *stream) {
    if (!it || !pcg_state) return iter_fail(JOKER_EINVAL, "joker_iter_admit: NULL argument");
    if (slot < 0 || slot >= it->p.n_stars)
        return iter_fail(JOKER_EINVAL, "joker_iter_admit: slot out of range");
    int64_t cap, cstride; const double *P, *E, *OM, *M0, *S; const float4 *ma, *mb; const float *ms;
    cache_internals(it->cache, &cap, &P, &E, &OM, &M0, &S, &cstride, &ma, &mb, &ms);
    if (budget <= 0 || it->p.lib_row0 + budget > cap)
        return iter_fail(JOKER_ERANGE, "joker_iter_admit: budget outside the cache");
    if (n_requested <= 0 || n_requested > it->p.max_req)
        return iter_fail(JOKER_ERANGE, "joker_iter_admit: n_requested outside [1, max_req]");
    if (init_batch <= 0 || init_batch > budget)
        return iter_fail(JOKER_EINVAL, "Prior sample library not big enough! For iterative "
                                       "sampling, you have to have at least growth_factor * "
                                       "n_requested_samples samples in the library.");
    if (pool_off < 0 || pool_off + budget > it->pool)
        return iter_fail(JOKER_ERANGE, "joker_iter_admit: pool range outside the pool");
    iter_admit_kernel<<<1, 1, 0, (cudaStream_t)stream>>>(
        it->p, it->max_key, it->bound_key, slot, budget, n_requested, init_batch, pool_off,
        pcg_state[0], pcg_state[1], pcg_state[2], pcg_state[3]);
    count_launch();
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return iter_fail(JOKER_ECUDA, cudaGetErrorString(e));
    return JOKER_OK;
}

extern "C" int joker_iter_create_pool(joker_iter **out, const joker_stars *stars,
                                      const joker_cache *cache, int precision, int64_t lib_row0,
                                      int64_t pool_samples, int max_requested,
                                      double safety_factor, int maxiter, int chunk) {
    return iter_alloc(out, stars, cache, precision, lib_row0, pool_samples, max_requested,
                      safety_factor, maxiter, chunk, "joker_iter_create_pool");
}

extern "C" int joker_iter_create(joker_iter **out, const joker_stars *stars,
                                 const joker_cache *cache, int precision, int64_t lib_row0,
                                 int64_t lib_size, int n_requested, int64_t init_batch,
                                 double safety_factor, int maxiter, const uint64_t *pcg_states,
                                 int chunk) {
    if (!pcg_states || !stars) return iter_fail(JOKER_EINVAL, "joker_iter_create: NULL argument");
    int n_stars = 0;
    {
        const StarRec *r; const double *a; const float *b; int L, jit; int *q;
        stars_internals(stars, &r, &a, &b, &n_stars, &L, &jit, &q);
    }
    int64_t cap, cstride; const double *P, *E, *OM, *M0, *S; const float4 *ma, *mb; const float *ms;
    cache_internals(cache, &cap, &P, &E, &OM, &M0, &S, &cstride, &ma, &mb, &ms);
    if (lib_row0 < 0 || lib_size <= 0 || lib_row0 + lib_size > cap)
        return iter_fail(JOKER_ERANGE, "joker_iter_create: library rows outside the cache");
    if (n_requested <= 0 || init_batch <= 0)
        return iter_fail(JOKER_EINVAL, "joker_iter_create: bad schedule parameters");
    if (init_batch > lib_size)
        return iter_fail(JOKER_EINVAL, "Prior sample library not big enough! For iterative "
                                       "sampling, you have to have at least growth_factor * "
                                       "n_requested_samples samples in the library.");
    joker_iter *it = nullptr;
    int rc = iter_alloc(&it, stars, cache, precision, lib_row0, lib_size * n_stars, n_requested,
                        safety_factor, maxiter, chunk, "joker_iter_create");
    if (rc != JOKER_OK) return rc;
    for (int s = 0; s < n_stars; ++s) {
        rc = joker_iter_admit(it, s, lib_size, n_requested, init_batch, (int64_t)s * lib_size,
                              pcg_states + 4 * (size_t)s, nullptr);
        if (rc != JOKER_OK) {
            joker_iter_destroy(it);
            return rc;
        }
    }
    if (cudaDeviceSynchronize() != cudaSuccess) {
        joker_iter_destroy(it);
        return iter_fail(JOKER_ECUDA, "joker_iter_create: admission failed");
    }
    *out = it;
    return JOKER_OK;
}

extern "C" int joker_iter_set_round_budget(joker_iter *it, int64_t samples) {
    if (!it) return iter_fail(JOKER_EINVAL, "joker_iter_set_round_budget: NULL handle");
    if (samples < 0) return iter_fail(JOKER_EINVAL, "joker_iter_set_round_budget: negative budget");
    it->p.round_budget = samples;
    return JOKER_OK;
}

extern "C" int joker_iter_destroy(joker_iter *it) {
    if (!it) return JOKER_OK;
    cudaFree(it->base);
    delete it;
    return JOKER_OK;
}

// One round.  Launches only (capturable into a CUDA graph).
extern "C" int joker_iter_round(joker_iter *it, void *stream) {
    if (!it) return iter_fail(JOKER_EINVAL, "joker_iter_round: NULL handle");
    cudaStream_t st = (cudaStream_t)stream;
    const bool mixed = it->precision != JOKER_FP64;
    iter_plan_kernel<<<1, 1024, 0, st>>>(it->p, mixed ? 1 : 0);
    count_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return iter_fail(JOKER_ECUDA, cudaGetErrorString(e));
    // ln L over the planned items
    const StarRec *recs; const double *ep64; const float *ep32; int n_stars, L, jit; int *queue;
    stars_internals(it->stars, &recs, &ep64, &ep32, &n_stars, &L, &jit, &queue);
    int64_t cap, cstride; const double *P, *E, *OM, *M0, *S; const float4 *ma, *mb; const float *ms;
    cache_internals(it->cache, &cap, &P, &E, &OM, &M0, &S, &cstride, &ma, &mb, &ms);
    LnlArgs a;
    memset(&a, 0, sizeof a);
    a.stars = recs; a.ep64 = ep64; a.ep32 = ep32;
    a.P = P; a.e = E; a.om = OM; a.M0 = M0; a.s = S; a.stride = cstride;
    a.mx_a = ma; a.mx_b = mb; a.mx_s2 = ms;
    a.items = it->p.items;
    a.n_items = (int)it->items_cap;
    a.n_items_dev = it->p.n_items;
    a.queue = it->queue;
    a.lnl = it->lnl;
    a.max_key = it->max_key;
    if (mixed) {
        a.err = it->err;
        a.bound_key = it->bound_key;
        a.err_c0 = mixed_err_c0();
        // samples out of reach of the maximum after their last epoch keep an
        // FP32 ln L and an infinite bound (the acceptance rejects them); the
        // maximum only grows over the rounds, so they stay out of reach
        a.oor_tail = it->precision == JOKER_MIXED_FAST;
    }
    if ((e = cudaMemsetAsync(it->queue, 0, sizeof(int), st)) != cudaSuccess ||
        (e = launch_lnl(it->precision, L, jit != 0, a, 128, st)) != cudaSuccess)
        return iter_fail(JOKER_ECUDA, cudaGetErrorString(e));
    // acceptance over every active star's prefix (grid-stride over the
    // device-counted blocks)
    AcceptArgs c;
    memset(&c, 0, sizeof c);
    if (mixed) {
        c.err = it->err;
        c.bound_key = it->bound_key;
        c.exact_key = it->p.exact_key;
        c.stars = recs;
        c.ep64 = ep64;
        c.ep32 = ep32;
        c.err_c0 = mixed_err_c0();
        c.P = P; c.E = E; c.OM = OM; c.M0 = M0; c.S = S;
        c.stride = cstride;
        c.L = L;
        c.jit = jit;
        c.n_refined = it->n_refined;
        c.write_max = 1;
        c.amb_words = it->amb;
        c.flag_list = it->flag_list;
        c.flag_count = it->flag_count;
        c.flag_cap = it->flag_cap;
        c.max_key = it->p.exact_key;
    } else {
        c.max_key = it->max_key;
    }
    c.segs = it->p.segs;
    c.blk_base = it->p.blk_base;
    c.total_blocks_dev = it->p.total_blocks;
    c.n_segs = it->p.n_stars;
    c.lnl = it->lnl;
    c.u_source = JOKER_U_PCG64;
    c.words = it->words;
    c.blk_count = it->blk_count;
    c.out_idx = it->out_idx;
    c.out_lnl = it->out_lnl;
    c.count = it->counts;
    // fixed grid: enough CTAs to cover the device, blocks looped in-kernel
    const int64_t grid = std::min<int64_t>(it->max_blocks, 152 * 8);
    if ((e = launch_accept(c, grid, st, false)) != cudaSuccess)
        return iter_fail(JOKER_ECUDA, cudaGetErrorString(e));
    iter_update_kernel<<<(n_stars + 255) / 256, 256, 0, st>>>(it->p);
    count_launch();
    if ((e = cudaGetLastError()) != cudaSuccess) return iter_fail(JOKER_ECUDA, cudaGetErrorString(e));
    return JOKER_OK;
}

// Device pointers of the results for the caller to copy: per star the state
// row (8 int64: start, n_process, n_evals, n_good, done, rounds, uniforms
// drawn, 0), the first n_requested accepted indices and their ln L, and the
// number of finished stars.
extern "C" int joker_iter_outputs(const joker_iter *it, int64_t **d_state, int64_t **d_idx,
                                  double **d_lnl, int **d_done, uint64_t **d_n_refined) {
    if (!it) return iter_fail(JOKER_EINVAL, "joker_iter_outputs: NULL handle");
    if (d_state) *d_state = it->p.state;
    if (d_idx) *d_idx = it->out_idx;
    if (d_lnl) *d_lnl = it->out_lnl;
    if (d_done) *d_done = it->p.done_count;
    if (d_n_refined) *d_n_refined = (uint64_t *)it->n_refined;
    return JOKER_OK;
}

// Synchronous copy of the results to host arrays (any may be NULL): the state
// rows (n_stars x 8), the accepted indices and their ln L (n_stars x
// n_requested) and the finished-star count.
extern "C" int joker_iter_read_async(const joker_iter *it, int64_t *h_state, const int *slots,
                                     int n_slots, int64_t *h_idx, void *stream) {
    if (!it) return iter_fail(JOKER_EINVAL, "joker_iter_read_async: NULL handle");
    if (n_slots < 0 || (n_slots > 0 && (!slots || !h_idx)))
        return iter_fail(JOKER_EINVAL, "joker_iter_read_async: bad slot list");
    const size_t n = (size_t)it->p.n_stars, r = (size_t)it->p.max_req;
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = cudaSuccess;
    if (h_state)
        e = cudaMemcpyAsync(h_state, it->p.state, 8 * n * ST_FIELDS, cudaMemcpyDeviceToHost, st);
    for (int k = 0; k < n_slots && e == cudaSuccess; ++k) {
        if (slots[k] < 0 || (size_t)slots[k] >= n)
            return iter_fail(JOKER_EINVAL, "joker_iter_read_async: slot outside the table");
        e = cudaMemcpyAsync(h_idx + (size_t)k * r, it->out_idx + (size_t)slots[k] * r, 8 * r,
                            cudaMemcpyDeviceToHost, st);
    }
    if (e != cudaSuccess) return iter_fail(JOKER_ECUDA, cudaGetErrorString(e));
    return JOKER_OK;
}

extern "C" int joker_iter_read(const joker_iter *it, int64_t *h_state, int64_t *h_idx,
                               double *h_lnl, int *h_done, uint64_t *h_n_refined) {
    if (!it) return iter_fail(JOKER_EINVAL, "joker_iter_read: NULL handle");
    const size_t n = (size_t)it->p.n_stars, r = (size_t)it->p.max_req;
    cudaError_t e = cudaSuccess;
    if (h_done && e == cudaSuccess) e = cudaMemcpy(h_done, it->p.done_count, 4, cudaMemcpyDeviceToHost);
    if (h_state && e == cudaSuccess)
        e = cudaMemcpy(h_state, it->p.state, 8 * n * ST_FIELDS, cudaMemcpyDeviceToHost);
    if (h_idx && e == cudaSuccess) e = cudaMemcpy(h_idx, it->out_idx, 8 * n * r, cudaMemcpyDeviceToHost);
    if (h_lnl && e == cudaSuccess) e = cudaMemcpy(h_lnl, it->out_lnl, 8 * n * r, cudaMemcpyDeviceToHost);
    if (h_n_refined && e == cudaSuccess)
        e = cudaMemcpy(h_n_refined, it->n_refined, 8, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return iter_fail(JOKER_ECUDA, cudaGetErrorString(e));
    return JOKER_OK;
}
