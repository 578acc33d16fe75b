// Prior samples drawn on the device, straight into a prior cache -- the
// producer of the reference's prior cache (JokerPrior.sample,
// thejoker/prior.py:297-407, with UniformLog / Kipping13Global of
// thejoker/distributions.py:19-28, 171-176) without the host draw, the
// HDF5 round trip and the upload.
//
// Random numbers: Philox4x32-10 (J. K. Salmon, M. A. Moraes, R. O. Dror and
// D. E. Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC11, 2011), a
// counter-based generator: sample g's draws come from counters
// (g_lo, g_hi, block, STREAM_TAG) under key (seed_lo, seed_hi), so every
// sample is reproducible from (seed, g) whatever the launch shape.  Each
// block yields two 64-bit halves, each one uniform: a double
// u = (x >> 11) 2^-53 for P and the angles, a float with 24 significant bits
// for the rest.  Per sample, in order: u_P, u_omega, u_M0, [one Box-Muller
// pair for ln s], then the two gamma variates of the beta draw.
//   P     = exp(ln P_min + u_P (ln P_max - ln P_min))          (FP64)
//   omega = 2 pi u_omega,  M0 = 2 pi u_M0                      (FP64)
//   e     = X / (X + Y),  X ~ Gamma(alpha), Y ~ Gamma(beta)   (Marsaglia and
//           Tsang, ACM TOMS 26, 2000; shape < 1 through
//           Gamma(a) = Gamma(a + 1) U^(1/a))                   (FP32)
//   s     = s_value, or exp(s_mu + s_sigma z)                  (FP32)
// The beta and log-normal draws run in FP32: they are random draws whose
// distribution FP32 rounding does not change measurably, and FP64 (1/74 of
// the FP32 rate here) made them the bound of the kernel.
#include "joker_internal.cuh"
#include "joker_math.cuh"

namespace joker {

namespace {
constexpr uint32_t PH_M0 = 0xD2511F53u, PH_M1 = 0xCD9E8D57u;
constexpr uint32_t PH_W0 = 0x9E3779B9u, PH_W1 = 0xBB67AE85u;
constexpr uint32_t STREAM_TAG = 0x4A6F6B72u;
constexpr int GAMMA_MAX_TRIES = 64;
}  // namespace

__host__ __device__ __forceinline__ void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
    for (int r = 0; r < 10; ++r) {
        const uint64_t p0 = (uint64_t)PH_M0 * c[0], p1 = (uint64_t)PH_M1 * c[2];
        const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0, n1 = (uint32_t)p1;
        const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1, n3 = (uint32_t)p0;
        c[0] = n0; c[1] = n1; c[2] = n2; c[3] = n3;
        k0 += PH_W0;
        k1 += PH_W1;
    }
}

// Sequential uniforms of one sample.
struct SampleRng {
    uint32_t g_lo, g_hi, k0, k1, block;
    uint64_t spare;
    bool have_spare;

    __device__ void init(uint64_t seed, uint64_t g) {
        g_lo = (uint32_t)g; g_hi = (uint32_t)(g >> 32);
        k0 = (uint32_t)seed; k1 = (uint32_t)(seed >> 32);
        block = 0;
        have_spare = false;
    }
    // the next 64-bit half of the sample's Philox stream
    __device__ uint64_t bits() {
        if (have_spare) { have_spare = false; return spare; }
        uint32_t c[4] = {g_lo, g_hi, block++, STREAM_TAG};
        philox4x32_10(c, k0, k1);
        spare = ((uint64_t)c[3] << 32) | c[2];
        have_spare = true;
        return ((uint64_t)c[1] << 32) | c[0];
    }
    __device__ double uniform() { return (double)(bits() >> 11) * 0x1.0p-53; }
    // A uniform float in (0, 1): the 24 bits of x / 2^64 below its leading
    // one, so the resolution follows the magnitude (down to 2^-64) and
    // log u reaches -44 (a Box-Muller normal is not cut off at 5.8 sigma).
    // Integer operations only.
    __device__ float uniform_f() {
        const uint64_t x = bits();
        if (x == 0) return 0x1.0p-65f;
        const int lz = __clzll(x);
        const uint32_t m = (uint32_t)((x << lz) >> 40);
        return __uint_as_float(((uint32_t)(126 - lz) << 23) | (m & 0x7fffffu));
    }
    // standard normal (Box-Muller in FP32; the second variate of the pair is dropped)
    __device__ float normal_f() {
        const float u1 = uniform_f();
        const float u2 = uniform_f();
        float s, c;
        sincospif(2.0f * u2, &s, &c);
        return sqrtf(-2.0f * logf(u1)) * c;
    }
    // Gamma(a, 1) in FP32, a > 0; *ok = false if the rejection loop ran out
    // of tries
    __device__ float gamma_f(float a, bool *ok) {
        const bool boost = a < 1.0f;
        const float k = boost ? a + 1.0f : a;
        const float d = k - 1.0f / 3.0f, c = 1.0f / sqrtf(9.0f * d);
        float v = 0.0f;
        bool got = false;
        for (int t = 0; t < GAMMA_MAX_TRIES && !got; ++t) {
            const float x = normal_f();
            const float w = fmaf(c, x, 1.0f);
            if (w <= 0.0f) continue;
            v = w * w * w;
            const float u = uniform_f();
            const float x2 = x * x;
            got = (u < 1.0f - 0.0331f * x2 * x2) ||
                  (logf(u) < 0.5f * x2 + d * (1.0f - v + logf(v)));
        }
        if (!got) *ok = false;
        float g = d * v;
        if (boost) g *= powf(uniform_f(), 1.0f / a);
        return g;
    }
};

__global__ void prior_sample_kernel(joker_prior_spec spec, uint64_t seed, int64_t first_index,
                                    int64_t n, int64_t row0, double *P, double *E, double *OM,
                                    double *M0, double *S, float4 *mx_a, float4 *mx_b,
                                    float *mx_s2, double *packed, int *bad) {
    const double lpmin = log(spec.P_min), lspan = log(spec.P_max) - lpmin;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        SampleRng rng;
        rng.init(seed, (uint64_t)(first_index + i));
        const double p = exp(fma(rng.uniform(), lspan, lpmin));
        const double om = rng.uniform() * TWO_PI_D;
        const double m0 = rng.uniform() * TWO_PI_D;
        double s = spec.s_value;
        if (spec.s_kind == JOKER_S_LOGNORMAL)
            s = (double)expf(fmaf((float)spec.s_sigma, rng.normal_f(), (float)spec.s_mu));
        bool ok = true;
        const float x = rng.gamma_f((float)spec.e_alpha, &ok);
        const float y = rng.gamma_f((float)spec.e_beta, &ok);
        double e = (double)(x / (x + y));
        if (!ok || !(e >= 0.0 && e < 1.0)) {
            atomicAdd(bad, 1);
            e = e >= 1.0 ? 0x1.fffffffffffffp-1 : (e >= 0.0 ? e : 0.0);
        }
        const int64_t r = row0 + i;
        P[r] = p; E[r] = e; OM[r] = om; M0[r] = m0; S[r] = s;
        float4 pa, pb;
        float s2;
        prepare_sample(p, e, om, m0, s, pa, pb, s2);
        mx_a[r] = pa;
        mx_b[r] = pb;
        mx_s2[r] = s2;
        if (packed) {
            double *q = packed + i * 5;
            q[0] = p; q[1] = e; q[2] = om; q[3] = m0; q[4] = s;
        }
    }
}

cudaError_t launch_prior_sample(const joker_prior_spec &spec, uint64_t seed, int64_t first_index,
                                int64_t n, int64_t row0, double *P, double *E, double *OM,
                                double *M0, double *S, float4 *mx_a, float4 *mx_b, float *mx_s2,
                                double *packed, int *bad, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    int64_t blocks = (n + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    prior_sample_kernel<<<(int)blocks, 256, 0, st>>>(spec, seed, first_index, n, row0, P, E, OM,
                                                     M0, S, mx_a, mx_b, mx_s2, packed, bad);
    count_launch();
    return cudaGetLastError();
}

}  // namespace joker
