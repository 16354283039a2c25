// Device-side building blocks shared by the engine kernels: complex
// arithmetic over float/double, Philox4x32-10, uniform mapping, block
// reductions and the job descriptor passed to every kernel.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/gpvmc_gb300.h"

namespace gv {

template <typename T>
struct alignas(2 * sizeof(T)) cx {
    T x, y;
};

template <typename T>
__host__ __device__ __forceinline__ cx<T> mk(T a, T b) { return cx<T>{a, b}; }
template <typename T>
__host__ __device__ __forceinline__ cx<T> operator+(cx<T> a, cx<T> b) { return {a.x + b.x, a.y + b.y}; }
template <typename T>
__host__ __device__ __forceinline__ cx<T> operator-(cx<T> a, cx<T> b) { return {a.x - b.x, a.y - b.y}; }
template <typename T>
__host__ __device__ __forceinline__ cx<T> operator*(cx<T> a, cx<T> b)
{
    return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
template <typename T>
__host__ __device__ __forceinline__ cx<T> operator*(cx<T> a, T s) { return {a.x * s, a.y * s}; }
template <typename T>
__host__ __device__ __forceinline__ T norm2(cx<T> a) { return a.x * a.x + a.y * a.y; }
template <typename T>
__host__ __device__ __forceinline__ cx<T> cinv(cx<T> a)
{
    T d = a.x * a.x + a.y * a.y;
    return {a.x / d, -a.y / d};
}
template <typename T>
__host__ __device__ __forceinline__ cx<T> cneg(cx<T> a) { return {-a.x, -a.y}; }
// a += b * c (complex multiply-accumulate)
template <typename T>
__device__ __forceinline__ void cmac(cx<T>& a, cx<T> b, cx<T> c)
{
    a.x = fma(b.x, c.x, a.x);
    a.x = fma(-b.y, c.y, a.x);
    a.y = fma(b.x, c.y, a.y);
    a.y = fma(b.y, c.x, a.y);
}
// Product rounded like the host's non-contracted (ac - bd, ad + bc).
__device__ __forceinline__ cx<double> cmul_rn(cx<double> a, cx<double> b)
{
    return {__dsub_rn(__dmul_rn(a.x, b.x), __dmul_rn(a.y, b.y)),
            __dadd_rn(__dmul_rn(a.x, b.y), __dmul_rn(a.y, b.x))};
}
__device__ __forceinline__ cx<float> cmul_rn(cx<float> a, cx<float> b)
{
    return {__fsub_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)),
            __fadd_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x))};
}

template <typename T>
__device__ __forceinline__ cx<double> to_d(cx<T> a) { return {double(a.x), double(a.y)}; }

// Philox4x32-10 (Salmon et al., SC'11).
__host__ __device__ __forceinline__ void philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                                       uint32_t k0, uint32_t k1, uint32_t out[4])
{
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
#ifdef __CUDA_ARCH__
        uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
        uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
#else
        uint64_t p0 = uint64_t(0xD2511F53u) * c0, p1 = uint64_t(0xCD9E8D57u) * c2;
        uint32_t hi0 = uint32_t(p0 >> 32), lo0 = uint32_t(p0), hi1 = uint32_t(p1 >> 32), lo1 = uint32_t(p1);
#endif
        uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c1 = lo1; c3 = lo0; c0 = n0; c2 = n2;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

// 52 random bits -> (m + 1/2) * 2^-52, exactly representable, in (0, 1).
__host__ __device__ __forceinline__ double u01(uint32_t a, uint32_t b)
{
    uint64_t m = ((uint64_t(a) << 20) ^ uint64_t(b >> 12)) & ((uint64_t(1) << 52) - 1);
    return (double(m) + 0.5) * (1.0 / 4503599627370496.0);
}

// 52 random bits of a uniform (the integer m in (m + 1/2) * 2^-52).
__host__ __device__ __forceinline__ uint64_t u52(uint32_t a, uint32_t b)
{
    return ((uint64_t(a) << 20) ^ uint64_t(b >> 12)) & ((uint64_t(1) << 52) - 1);
}

// floor(double(n) * u) for u = (m + 1/2) 2^-52 and 1 <= n < 2^10, computed in
// integers with the IEEE double product's round-to-nearest-even, so that it
// equals the reference's size_t(n * RanGen::uniform()) bit for bit
// (LatticeStepper.cpp:45) without touching the FP64 pipe.
__host__ __device__ __forceinline__ int scaled_floor(uint32_t n, uint64_t m)
{
    const uint64_t X = uint64_t(n) * (2 * m + 1);   // exact product n (2m+1), < 2^63
#ifdef __CUDA_ARCH__
    const int b = 64 - __clzll((long long)X);
#else
    const int b = 64 - __builtin_clzll(X);
#endif
    if (b <= 53) return int(X >> 53);               // exactly representable
    const int s = b - 53;
    uint64_t q = X >> s;
    const uint64_t r = X & ((uint64_t(1) << s) - 1), half = uint64_t(1) << (s - 1);
    if (r > half || (r == half && (q & 1))) ++q;    // round half to even
    return int((q << s) >> 53);
}

// Stream layout: counter {call_lo, call_hi, walker, stream}, key {seed_lo,
// seed_hi}; uniform k comes from call k/2 (words 0,1 for even k, 2,3 for odd).
__host__ __device__ __forceinline__ void philox_call(uint64_t seed, uint32_t walker, uint32_t stream,
                                                     uint64_t call, uint32_t out[4])
{
    philox4x32_10(uint32_t(call), uint32_t(call >> 32), walker, stream, uint32_t(seed),
                  uint32_t(seed >> 32), out);
}

__host__ __device__ __forceinline__ double uniform_at(uint64_t seed, uint32_t walker, uint32_t stream,
                                                      uint64_t k)
{
    uint32_t x[4];
    philox_call(seed, walker, stream, k >> 1, x);
    return (k & 1) ? u01(x[2], x[3]) : u01(x[0], x[1]);
}

// Exciton ProjHeis measurements of a mixed job summed in FP32 before one FP64
// add per H / O entry (a block of this many measurements per walker).
constexpr int kHoSlots = 32;

// Everything a kernel needs about a job (device pointers, sizes).
struct DevJob {
    int L, Ns, Nk, Nexc, W;
    int N[2], Nmax;
    int precision, channel;
    uint64_t seed;
    uint32_t walker_base;
    int reinv_every;
    const int32_t* nbr;        // Ns*4
    const int4* edges;         // 2*Ns edges (i, j, slot of j in nbr[i], slot of i in nbr[j]), creation order
    const cx<double>* phase64; // Ns*Nk
    const cx<float>* phase32;
    const cx<double>* coef64;  // W*2fl*2sub*Ns
    const cx<float>* coef32;
    void* Ai[2];               // W * N[fl]^2, row-major [particle][row]
    int16_t* fock;             // W*2*Ns: particle index at site or -1
    int16_t* part;             // W*2*Nmax: site of particle
    cx<double>* amp_m;         // W amplitude mantissa (|m| in [1,2) or 0)
    int32_t* amp_e;            // W amplitude base-2 exponent
    uint64_t* rng_next;        // W Metropolis uniform index
    unsigned long long* counts;// W*5
    int32_t* since_reinv;      // W accepted exchanges since the last re-inversion / drift check
    unsigned long long* checks;// W drift checks that did not need a re-inversion
    double* drift_seen;        // W largest sampled drift seen at a check
    int32_t* status;           // W
    cx<double>* pj;            // W*2
    int32_t* pj_n;
    cx<double>* sm;            // W
    int32_t* sm_n;
    double* ss;                // job-wide StatSpinStruct sums, compact: T (Ns*Ns complex) then
                               // Aud (Ns*Ns real) in a 10*Ns*Ns-double buffer
    int32_t* ss_n;
    uint32_t* occ;             // 2*Ns*ceil(W/32) occupation bitsets (tensor-core StatSpinStruct)
    float2* ss32;              // Ns*Ns FP32 staging sums of one tensor-core StatSpinStruct measurement
    double* track_sm;          // W*track_cap StagMagnTrack values
    double* track_lw;          // W*track_cap OverlapTrack log10 weights
    int32_t* track_n;          // W entries recorded
    int track_cap;
    cx<double>* scratch64;     // per-CTA FP64 N*N scratch for re-inversion (W*Nmax*Nmax)
    gv_trace* trace;
    int trace_walker;
    // Transverse-exciton channel only (null for the ground state).  The
    // wavefunction's Fock state per walker: Slater row (slot) f holds orbital
    // worb[f]; wslot[o] is the slot of orbital o or -1.  Channel state k
    // differs from the current one `cur` by one flavour-0 hop
    // exc_up[cur] -> exc_up[k] and one flavour-1 hop exc_dn[k] -> exc_dn[cur].
    int16_t* worb;             // W*2*Nmax
    int16_t* wslot;            // W*2*Ns
    const int16_t* exc_up;     // Nexc: flavour-0 upper-band orbital of state k
    const int16_t* exc_dn;     // Nexc: flavour-1 lower-band hole of state k
    int32_t* cur;              // W: current channel state (WaveFunction::m_c_exc)
    int32_t* wsign;            // W: sign of the wavefunction's Fock state (State::m_sign)
    double* sigma;             // W: state weight / |det_0 det_1|^2 = sum_k |ratio_k|^2
    void* gup;                 // W*N0*Nexc, GupT[f][k] = sum_p phi_{exc_up[k]}(x_p) (A0^-1)(p, f)
    void* gdn;                 // W*Nmax,    g[f] = sum_p phi_{exc_dn[cur]}(x_p) (A1^-1)(p, f)
    cx<double>* pjx;           // W*2*Nexc*Nexc ProjHeis H and O sums
    // Mixed exciton jobs: each measurement's FP32 factors (conj(a)/w, h, a; 3*Nexc
    // each) wait in one of kHoSlots slots per walker and are folded into pjx as a
    // block every kHoSlots measurements (null for FP64 jobs, which add at once).
    cx<float>* pxs;            // W*kHoSlots*3*Nexc
    int32_t* pxs_n;            // W: measurements waiting in pxs
    cx<float>* zbuf;          // W*N1*Nexc tensor-core Z[d][k] = sum_f GupT[f][k] phi_f(d) (mixed, or null)
    int wait_limit;            // polls before a bounded mbarrier wait of the tensor-core kernels gives up
    // Single-walker stepping (gv_job_trystep / gv_job_step, LatticeStepper::trystep / step):
    // when forced_walker >= 0 the streaming walk kernels run that walker only, take the
    // proposal (forced_v1, forced_v2) instead of drawing it and leave its Philox position
    // alone; forced_accept = 1 applies the move (LatticeStepper::step), 0 only evaluates it
    // into the trace record and writes nothing back; forced_khop >= 0 picks that channel
    // state instead of the arg-max.
    int forced_walker, forced_v1, forced_v2, forced_accept, forced_khop;
};

// Amplitude kept as (complex mantissa, base-2 exponent); renormalised
// exactly by powers of two.
__device__ __forceinline__ void amp_normalise(cx<double>& m, int& e)
{
    double a = fmax(fabs(m.x), fabs(m.y));
    if (a == 0.0 || !isfinite(a)) return;
    int k;
    frexp(a, &k);
    m.x = ldexp(m.x, -k);
    m.y = ldexp(m.y, -k);
    e += k;
}

template <int NT>
__device__ __forceinline__ double block_sum_d(double v, double* red)
{
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0;
#pragma unroll
    for (int w = 0; w < NT / 32; ++w) s += red[w];
    return s;
}

}  // namespace gv
