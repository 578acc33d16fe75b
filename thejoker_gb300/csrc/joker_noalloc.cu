// joker_accept_noalloc: the acceptance pass for callers that may not allocate
// device memory.
//
// Some callers of this library cannot call cudaMalloc:
// - A serving loop with per-request deadlines. cudaMalloc may synchronise the
//   whole device and has unbounded latency, so such a loop allocates everything
//   once at start-up and nothing afterwards.
// - A host framework whose caching allocator has already reserved the device's
//   free memory. A raw cudaMalloc from a plugin there fails, or fragments the
//   pool that framework manages.
// For them this file keeps the pass's scratch space (the per-CTA counts, the
// accepted-sample bit masks and the copied segment table) in one file-scope
// device array of fixed size, instead of a caller-supplied workspace.
//
// The array, ACC_SCRATCH_BYTES = 2,220,288 bytes, is static device data of
// this file's module.  Under lazy module loading (the CUDA default since 12.2)
// that module, and with it the array's device memory, is loaded on a device at
// the first lookup of the array there.  So each device needs one warm-up call
// at start-up, with that device current and before any stream capture: a call
// with n_segs = 0 does the lookup and loads the pass's kernels, and runs
// nothing.  A first call that does real work does the same set-up itself, so
// if it comes first it is the call that loads the module and takes the
// memory.  From then on the device holds the array until the process exits.
// Its limits are:
// - at most JOKER_NOALLOC_MAX_SEGS segments;
// - at most JOKER_NOALLOC_MAX_BLOCKS blocks of 8192 samples, counted per
//   segment and rounded up (about 2^24 samples in all).
// A call above either limit is rejected with JOKER_ERANGE, and nothing runs.
//
// Every call shares the one array, and the array keeps the last call's
// contents. Each word a call reads is first written by that same call (the
// mark kernel writes every mask word and every CTA count of its blocks before
// the scan and emit kernels read them), so nothing needs to be cleared. Calls
// whose work overlaps on the GPU race on the array: two streams must not run
// this entry point at the same time on one device.
//
// Each call copies the segment table (and its block offsets, from the
// stack) into the array with cudaMemcpyAsync on the caller's stream.  From
// pageable memory the copy is staged before the call returns; a segment table
// in pinned memory is read by the copy engine later, so it must stay unchanged
// until the stream has passed the call.
//
// The array's device address is looked up once per device and kept for the
// life of the process.  After cudaDeviceReset the module may be reloaded at
// another address, so this entry point must not be used on a device after a
// reset of that device.
#include <cstdio>
#include <cstring>
#include <mutex>
#include "joker_internal.cuh"

namespace joker {
cudaError_t launch_accept(const AcceptArgs &a, int64_t total_blocks, cudaStream_t st,
                          bool max_given = false);
cudaError_t accept_preload();
int64_t accept_blocks(const joker_accept_seg *segs, int n_segs, int64_t *blk_base_host);
void set_last_error(const char *msg);
}  // namespace joker

using namespace joker;

namespace {

constexpr int MAX_SEGS = JOKER_NOALLOC_MAX_SEGS;
constexpr int64_t MAX_BLOCKS = JOKER_NOALLOC_MAX_BLOCKS;
constexpr int64_t WORDS_PER_BLOCK = 256;     // 32-bit masks per 8192-sample block

constexpr size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }
constexpr size_t OFF_SEGS = 0;
constexpr size_t OFF_BASE = OFF_SEGS + align_up(sizeof(joker_accept_seg) * MAX_SEGS);
constexpr size_t OFF_COUNT = OFF_BASE + align_up(sizeof(int64_t) * (MAX_SEGS + 1));
constexpr size_t OFF_WORDS = OFF_COUNT + align_up(sizeof(int64_t) * MAX_BLOCKS);
constexpr size_t ACC_SCRATCH_BYTES = OFF_WORDS + align_up(4 * WORDS_PER_BLOCK * MAX_BLOCKS);
static_assert(ACC_SCRATCH_BYTES == 2220288, "scratch size changed: update the comments");

constexpr int MAX_DEVICES = 64;

std::mutex g_mutex;
unsigned char *g_scratch_addr[MAX_DEVICES] = {};

}  // namespace

// The scratch space itself.  Host code must never pass this name to a kernel:
// on the host it only stands for the symbol, not a device address.
static __device__ __align__(256) unsigned char g_accept_scratch[ACC_SCRATCH_BYTES];

// Device address of g_accept_scratch on the current device, looked up once
// per device; the first lookup also loads the pass's kernels, so that later
// calls load no module.
static cudaError_t scratch_address(unsigned char **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= MAX_DEVICES) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_mutex);
    if (g_scratch_addr[dev] == nullptr) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_accept_scratch);
        if (e != cudaSuccess) return e;
        e = accept_preload();
        if (e != cudaSuccess) return e;
        g_scratch_addr[dev] = static_cast<unsigned char *>(p);
    }
    *out = g_scratch_addr[dev];
    return cudaSuccess;
}

static int noalloc_fail(int code, const char *msg) {
    set_last_error(msg);
    return code;
}

static int noalloc_cuda_fail(const char *what, cudaError_t e) {
    char buf[256];
    snprintf(buf, sizeof buf, "joker_accept_noalloc: %s: %s", what, cudaGetErrorString(e));
    set_last_error(buf);
    return JOKER_ECUDA;
}

extern "C" int joker_accept_noalloc(const joker_accept_seg *segs, int n_segs,
                                    const double *d_lnl, const uint64_t *d_max_key,
                                    int u_source, const double *d_u, int64_t *d_out_idx,
                                    double *d_out_lnl, int64_t *d_count, void *stream) {
    // set-up first, so that a call with no segments is the warm-up call
    unsigned char *scratch = nullptr;
    cudaError_t e = scratch_address(&scratch);
    if (e != cudaSuccess) return noalloc_cuda_fail("cudaGetSymbolAddress", e);
    if (n_segs <= 0) return JOKER_OK;
    if (!segs || !d_lnl || !d_max_key || !d_out_idx || !d_count)
        return noalloc_fail(JOKER_EINVAL, "joker_accept_noalloc: NULL argument");
    if (u_source != JOKER_U_ARRAY && u_source != JOKER_U_PCG64)
        return noalloc_fail(JOKER_EINVAL, "joker_accept_noalloc: unknown u_source");
    if (u_source == JOKER_U_ARRAY && !d_u)
        return noalloc_fail(JOKER_EINVAL, "joker_accept_noalloc: d_u is NULL");
    if (n_segs > MAX_SEGS)
        return noalloc_fail(JOKER_ERANGE,
                            "joker_accept_noalloc: more segments than JOKER_NOALLOC_MAX_SEGS");
    for (int i = 0; i < n_segs; ++i)
        if (segs[i].n < 0 || segs[i].max_out < 0 || segs[i].lnl_off < 0 || segs[i].max_slot < 0)
            return noalloc_fail(JOKER_EINVAL, "joker_accept_noalloc: negative segment field");
    int64_t base[MAX_SEGS + 1];                    // on the stack: no heap use either
    const int64_t nb = accept_blocks(segs, n_segs, base);
    if (nb > MAX_BLOCKS)
        return noalloc_fail(JOKER_ERANGE,
                            "joker_accept_noalloc: more 8192-sample blocks than "
                            "JOKER_NOALLOC_MAX_BLOCKS (about 2^24 samples)");
    cudaStream_t st = (cudaStream_t)stream;
    joker_accept_seg *d_segs = reinterpret_cast<joker_accept_seg *>(scratch + OFF_SEGS);
    int64_t *d_base = reinterpret_cast<int64_t *>(scratch + OFF_BASE);
    // pageable host sources are staged before cudaMemcpyAsync returns, so the
    // stack copy of `base` may go out of scope afterwards
    e = cudaMemcpyAsync(d_segs, segs, sizeof(joker_accept_seg) * n_segs, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_base, base, sizeof(int64_t) * (n_segs + 1), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return noalloc_cuda_fail("cudaMemcpyAsync", e);
    AcceptArgs a;
    memset(&a, 0, sizeof a);
    a.segs = d_segs;
    a.blk_base = d_base;
    a.n_segs = n_segs;
    a.lnl = d_lnl;
    a.max_key = reinterpret_cast<const unsigned long long *>(d_max_key);
    a.u_source = u_source;
    a.u = d_u;
    a.words = reinterpret_cast<uint32_t *>(scratch + OFF_WORDS);
    a.blk_count = reinterpret_cast<int64_t *>(scratch + OFF_COUNT);
    a.out_idx = d_out_idx;
    a.out_lnl = d_out_lnl;
    a.count = d_count;
    e = launch_accept(a, nb, st);
    if (e != cudaSuccess) return noalloc_cuda_fail("launch", e);
    return JOKER_OK;
}
