// Ground-state Metropolis walk with both inverses resident in tensor memory
// (mixed precision, N <= 128).  Included by engine.cu after kernels.cuh.
//
// The streaming kernel (k_walk_gs) keeps the inverses in HBM and runs several
// walkers per SM to hide the latency of every proposal's row gather and every
// accepted move's read-modify-write; it settles at ~75% of the HBM copy
// bandwidth.  Here one CTA per SM owns one walker for a whole walk call and
// keeps both FP32 inverses in the SM's tensor memory (TMEM: 128 lanes x 512
// 32-bit columns = 256 KB): flavour g occupies columns [256 g, 256 g + 256),
// lane f holds row f of AiT (AiT[f][p] = (A^-1)(p, f)) with the real and
// imaginary part of particle p in columns 2p and 2p + 1.  HBM is touched once
// per walk call (load at entry, store at exit).  Warpgroup g (threads
// 128 g .. 128 g + 127; TMEM lane f = thread f of the warpgroup) serves flavour
// g; both flavours run concurrently:
//   proposal: thread f loads its lane's element of column c (one 2-column
//             load), forms (A^-1)(c, f) u_f and the warpgroup sums the
//             ratio r = sum_f (A^-1)(c, f) u_f  (linalg.cpp:297-303);
//   accept:   w = A^-1 u for every particle: each warp multiplies its 32 rows
//             by u_f and transposes-and-sums them across its lanes with
//             shuffles, the four warps' partial sums meet in shared memory;
//             then every lane updates its row,
//             AiT[f][p] -= (w_p - [p == c]) (A^-1)(c, f) / r  (linalg.cpp:402-573, rc = 1).
// Uniforms are drawn 32 steps at a time by one warp into shared memory (the
// Metropolis stream does not depend on the walk).  Same uniforms, decisions
// and formulas as k_walk_gs.
#pragma once

#include "kernels.cuh"

namespace gv {
namespace {

// ---- tensor memory (tcgen05): allocation and 32-lane access ----
__device__ __forceinline__ void tmem_alloc(uint32_t* dst_smem, uint32_t ncols)
{
    const uint32_t a = static_cast<uint32_t>(__cvta_generic_to_shared(dst_smem));
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(a), "r"(ncols) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tmem_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tmem_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }
// Thread i of a warp accesses lane (lane base of taddr) + i, columns [col, col + n);
// the wait takes the registers as operands so that no use is hoisted above it.
__device__ __forceinline__ void tmem_ld2(uint32_t taddr, uint32_t (&r)[2])
{
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x2.b32 {%0,%1}, [%2];" : "=r"(r[0]), "=r"(r[1]) : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld(uint32_t (&r)[2])
{
    asm volatile("tcgen05.wait::ld.sync.aligned;" : "+r"(r[0]), "+r"(r[1])::"memory");
}
__device__ __forceinline__ void tmem_ld64(uint32_t taddr, uint32_t (&r)[64])
{
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x64.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32,%33,%34,%35,%36,%37,%38,%39,%40,%41,%42,%43,%44,%45,%46,%47,%48,%49,%50,%51,%52,%53,%54,%55,%56,%57,%58,%59,%60,%61,%62,%63}, [%64];" : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31]), "=r"(r[32]), "=r"(r[33]), "=r"(r[34]), "=r"(r[35]), "=r"(r[36]), "=r"(r[37]), "=r"(r[38]), "=r"(r[39]), "=r"(r[40]), "=r"(r[41]), "=r"(r[42]), "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47]), "=r"(r[48]), "=r"(r[49]), "=r"(r[50]), "=r"(r[51]), "=r"(r[52]), "=r"(r[53]), "=r"(r[54]), "=r"(r[55]), "=r"(r[56]), "=r"(r[57]), "=r"(r[58]), "=r"(r[59]), "=r"(r[60]), "=r"(r[61]), "=r"(r[62]), "=r"(r[63]) : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld(uint32_t (&r)[64])
{
    asm volatile("tcgen05.wait::ld.sync.aligned;" : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]), "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]), "+r"(r[15]), "+r"(r[16]), "+r"(r[17]), "+r"(r[18]), "+r"(r[19]), "+r"(r[20]), "+r"(r[21]), "+r"(r[22]), "+r"(r[23]), "+r"(r[24]), "+r"(r[25]), "+r"(r[26]), "+r"(r[27]), "+r"(r[28]), "+r"(r[29]), "+r"(r[30]), "+r"(r[31]), "+r"(r[32]), "+r"(r[33]), "+r"(r[34]), "+r"(r[35]), "+r"(r[36]), "+r"(r[37]), "+r"(r[38]), "+r"(r[39]), "+r"(r[40]), "+r"(r[41]), "+r"(r[42]), "+r"(r[43]), "+r"(r[44]), "+r"(r[45]), "+r"(r[46]), "+r"(r[47]), "+r"(r[48]), "+r"(r[49]), "+r"(r[50]), "+r"(r[51]), "+r"(r[52]), "+r"(r[53]), "+r"(r[54]), "+r"(r[55]), "+r"(r[56]), "+r"(r[57]), "+r"(r[58]), "+r"(r[59]), "+r"(r[60]), "+r"(r[61]), "+r"(r[62]), "+r"(r[63])::"memory");
}
__device__ __forceinline__ void tmem_wait_ld(uint32_t (&r)[4])
{
    asm volatile("tcgen05.wait::ld.sync.aligned;" : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3])::"memory");
}
__device__ __forceinline__ void tmem_wait_ld(uint32_t (&r)[6])
{
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5])::"memory");
}
__device__ __forceinline__ void tmem_wait_ld(uint32_t (&r)[8])
{
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7])::"memory");
}
__device__ __forceinline__ void tmem_st64(uint32_t taddr, const uint32_t (&r)[64])
{
    asm volatile("tcgen05.st.sync.aligned.32x32b.x64.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32,%33,%34,%35,%36,%37,%38,%39,%40,%41,%42,%43,%44,%45,%46,%47,%48,%49,%50,%51,%52,%53,%54,%55,%56,%57,%58,%59,%60,%61,%62,%63,%64};" ::"r"(taddr), "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]), "r"(r[8]), "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15]), "r"(r[16]), "r"(r[17]), "r"(r[18]), "r"(r[19]), "r"(r[20]), "r"(r[21]), "r"(r[22]), "r"(r[23]), "r"(r[24]), "r"(r[25]), "r"(r[26]), "r"(r[27]), "r"(r[28]), "r"(r[29]), "r"(r[30]), "r"(r[31]), "r"(r[32]), "r"(r[33]), "r"(r[34]), "r"(r[35]), "r"(r[36]), "r"(r[37]), "r"(r[38]), "r"(r[39]), "r"(r[40]), "r"(r[41]), "r"(r[42]), "r"(r[43]), "r"(r[44]), "r"(r[45]), "r"(r[46]), "r"(r[47]), "r"(r[48]), "r"(r[49]), "r"(r[50]), "r"(r[51]), "r"(r[52]), "r"(r[53]), "r"(r[54]), "r"(r[55]), "r"(r[56]), "r"(r[57]), "r"(r[58]), "r"(r[59]), "r"(r[60]), "r"(r[61]), "r"(r[62]), "r"(r[63]) : "memory");
}
// barrier over one warpgroup (ids 1, 2; id 0 is __syncthreads)
__device__ __forceinline__ void wg_sync(int g) { asm volatile("bar.sync %0, 128;" ::"r"(1 + g) : "memory"); }

constexpr int kResThreads = 256;
constexpr int kResTmemCols = 512;                 // both flavours, 128 complex FP32 per lane each
constexpr size_t kResMinSmem = 116 * 1024;        // over half an SM's shared memory: one CTA per SM
constexpr int kResRngBatch = 32;
constexpr int kResSpec = 2;                       // proposals evaluated per barrier

struct ResLayout {
    size_t fock, part, nbr, sub, coef, red, wpart, w, rv, ru4, ru4d, racc, rq, rqp, nb, redm, tbase, total, used;
};

__host__ __device__ inline ResLayout res_layout(int Ns, int N, bool projheis)
{
    ResLayout l;
    size_t b = 0;
    auto al = [&](size_t x) { b = (b + 15) & ~size_t(15); size_t r = b; b += x; return r; };
    const size_t c = sizeof(cx<float>);
    l.fock = al(sizeof(int16_t) * 2 * Ns);
    l.part = al(sizeof(int16_t) * 2 * N);
    l.nbr = al(sizeof(int16_t) * 4 * Ns);
    l.sub = al(sizeof(int8_t) * Ns);
    l.coef = al(c * 4 * N);
    l.red = al(sizeof(float) * 2 * 16 * kResSpec);
    l.wpart = al(c * 2 * 4 * 128);
    l.w = al(c * 2 * 128);
    l.rv = al(sizeof(int16_t) * 2 * kResRngBatch);
    l.ru4 = al(sizeof(float) * kResRngBatch);
    l.ru4d = al(sizeof(double) * kResRngBatch);
    l.racc = al(sizeof(cx<float>) * 2 * kResRngBatch);   // accepted ratio pairs of the batch
    l.rq = al(projheis ? c * 4 * Ns : 16);
    l.rqp = al(projheis ? c * 2 * 4 * 4 * 128 : 16);   // [g][warp][slot][p] partial bond ratios
    l.nb = al(projheis ? sizeof(int32_t) * 2 * 4 * 128 : 16);   // [g][bond] particle, slot and site
    l.redm = al(sizeof(double) * 4 * (kResThreads / 32));
    l.tbase = al(sizeof(uint32_t));
    l.used = al(16);
    l.total = l.used < kResMinSmem ? kResMinSmem : l.used;
    return l;
}

// v[0..31] per lane -> lane l returns the sum over the warp's lanes of v[l]:
// a butterfly reduce-scatter in registers (at the step with offset o each
// lane keeps the half of its o-wide block that its lane bit selects, sends
// the other half to lane ^ o and adds what it receives): 31 complex shuffles
// per lane, no shared memory.
__device__ __forceinline__ cx<float> warp_reduce_scatter(cx<float> (&v)[32])
{
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        const bool hi = (lane & o) != 0;
#pragma unroll
        for (int t = 0; t < o; ++t) {
            const cx<float> keep = hi ? v[o + t] : v[t];
            cx<float> send = hi ? v[t] : v[o + t];
            send.x = __shfl_xor_sync(0xffffffffu, send.x, o);
            send.y = __shfl_xor_sync(0xffffffffu, send.y, o);
            v[t] = keep + send;
        }
    }
    return v[0];
}

__global__ void __launch_bounds__(kResThreads, 1) k_walk_gs_res(DevJob J, uint64_t nsteps, uint64_t s0, uint64_t meas,
                                                                int mask)
{
    extern __shared__ __align__(16) char smem[];
    using T = float;
    const int w = blockIdx.x;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (w >= J.W || J.status[w] != GV_OK) return;   // before any TMEM allocation
    const int Ns = J.Ns, N = J.N[0], L = J.L, Nk = J.Nk;
    const int NCH = (N + 31) / 32;                  // 32-particle column chunks
    const ResLayout lay = res_layout(Ns, N, (mask & GV_MEAS_PROJHEIS) != 0);
    int16_t* s_fock = reinterpret_cast<int16_t*>(smem + lay.fock);
    int16_t* s_part = reinterpret_cast<int16_t*>(smem + lay.part);
    int16_t* s_nbr = reinterpret_cast<int16_t*>(smem + lay.nbr);
    int8_t* s_sub = reinterpret_cast<int8_t*>(smem + lay.sub);
    cx<T>* s_coef = reinterpret_cast<cx<T>*>(smem + lay.coef);
    T* s_red = reinterpret_cast<T*>(smem + lay.red);
    cx<T>* s_wpart = reinterpret_cast<cx<T>*>(smem + lay.wpart);   // [g][warp][p]
    cx<T>* s_w = reinterpret_cast<cx<T>*>(smem + lay.w);           // [g][p]
    int16_t* s_rv = reinterpret_cast<int16_t*>(smem + lay.rv);     // [step][v1, v2]
    float* s_ru4 = reinterpret_cast<float*>(smem + lay.ru4);
    double* s_ru4d = reinterpret_cast<double*>(smem + lay.ru4d);
    cx<T>* s_racc = reinterpret_cast<cx<T>*>(smem + lay.racc);
    cx<T>* s_rq = reinterpret_cast<cx<T>*>(smem + lay.rq);
    cx<T>* s_rqp = reinterpret_cast<cx<T>*>(smem + lay.rqp);
    int32_t* s_nb = reinterpret_cast<int32_t*>(smem + lay.nb);
    double* s_redm = reinterpret_cast<double*>(smem + lay.redm);
    uint32_t* s_tbase = reinterpret_cast<uint32_t*>(smem + lay.tbase);

    if (warp == 0) tmem_alloc(s_tbase, kResTmemCols);
    for (int i = tid; i < 2 * Ns; i += kResThreads) s_fock[i] = J.fock[size_t(w) * 2 * Ns + i];
    for (int i = tid; i < 2 * N; i += kResThreads) {
        const int fl = i / N, p = i % N;
        s_part[i] = J.part[(size_t(w) * 2 + fl) * J.Nmax + p];
    }
    for (int i = tid; i < 4 * Ns; i += kResThreads) s_nbr[i] = int16_t(J.nbr[i]);
    for (int i = tid; i < Ns; i += kResThreads) s_sub[i] = int8_t(sublattice(i, L));
    {
        const cx<T>* cg = J.coef32 + size_t(w) * 4 * Ns;   // [fl][sub][orbital]
        for (int i = tid; i < 4 * N; i += kResThreads) {
            const int fl = i / (2 * N), sub = (i / N) & 1, f = i % N;
            s_coef[i] = cg[(size_t(fl) * 2 + sub) * Ns + 2 * f];
        }
    }
    tmem_fence_before();
    __syncthreads();
    tmem_fence_after();
    const uint32_t tbase = *s_tbase;
    const int g = tid >> 7;                       // warpgroup = flavour
    const int f = tid & 127;                      // TMEM lane = Slater row of this thread
    const uint32_t trow = tbase + ((uint32_t(warp & 3) * 32) << 16) + uint32_t(256 * g);
    cx<T>* Ag = ai_ptr<T>(J, g, w);
    // inverse of flavour g -> TMEM: lane f = row f of AiT (contiguous in HBM), zero padding
    for (int c = 0; c < NCH; ++c) {
        uint32_t r[64];
#pragma unroll
        for (int j = 0; j < 32; ++j) {
            const int p = 32 * c + j;
            cx<T> a = {0.f, 0.f};
            if (f < N && p < N) a = Ag[size_t(f) * N + p];
            r[2 * j] = __float_as_uint(a.x);
            r[2 * j + 1] = __float_as_uint(a.y);
        }
        tmem_st64(trow + 64 * c, r);
    }
    tmem_wait_st();
    tmem_fence_before();
    __syncthreads();
    tmem_fence_after();

    const cx<T>* phase = J.phase32;
    const cx<T>* cf = s_coef + g * 2 * N;         // this flavour's [sub][f]
    const uint32_t wid = J.walker_base + uint32_t(w);
    uint64_t k = J.rng_next[w];
    unsigned long long c_acc = 0, c_noop = 0, c_rej = 0;
    int since = J.since_reinv[w];
    cx<double> am = J.amp_m[w];
    int ae = J.amp_e[w];
    int status = GV_OK;
    int rbuf = 0;
    int nacc = 0;   // accepted ratio pairs waiting to be multiplied into the amplitude
    const WalkCtx<T> C = {&J, w, Ns, N, L, Nk, N, N, s_fock, s_part, s_nbr, s_coef, s_rq, s_redm,
                          phase, ai_ptr<T>(J, 0, w), ai_ptr<T>(J, 1, w)};
    // Proposals are evaluated kResSpec at a time: every thread forms its terms
    // of the next kb proposals' ratios (same inverse, same occupancy), one
    // barrier combines them, and the steps are then resolved in order until
    // the first accepted move, whose update invalidates the rest (they are
    // evaluated again, from the new inverse, in the next round).  A round
    // never crosses a uniform batch or a measurement step.
    // phase rows of both sites of the next round's proposals, fetched during the
    // current round (whichever site a proposal's particle moves to, its row is there)
    cx<T> pf[kResSpec][2];
    int pf_bi = -1;   // first proposal index of the prefetched rows, -1: none
    const bool measuring = meas != 0 && mask != 0;
    // steps from s to the next measuring step (0: s itself is measured)
    uint64_t to_meas = measuring ? (meas == 1 ? 0 : (meas - (s0 % meas)) % meas) : ~uint64_t(0);
    uint64_t s = 0;
    while (s < nsteps) {
        const int bi0 = int(s % kResRngBatch);
        if (bi0 == 0) {   // the next batch of proposals and accept uniforms (one lane per step)
            __syncthreads();   // every thread is done with the previous batch
            // the amplitude (FP64, off the per-step path): the previous batch's accepted ratios
            if (tid == 32) {
                for (int i = 0; i < nacc; ++i) {
                    am = am * (to_d(s_racc[2 * i]) * to_d(s_racc[2 * i + 1]));
                    amp_normalise(am, ae);
                }
            }
            nacc = 0;
            if (warp == 0 && s + lane < nsteps) {
                const uint64_t kl = k + 4 * (s + uint64_t(lane));
                uint32_t x[4], y[4];
                philox_call(J.seed, wid, 0, kl >> 1, x);
                philox_call(J.seed, wid, 0, (kl >> 1) + 1, y);
                const int v1 = scaled_floor(uint32_t(Ns), u52(x[0], x[1]));
                s_rv[2 * lane] = int16_t(v1);
                s_rv[2 * lane + 1] = s_nbr[v1 * 4 + int(u52(x[2], x[3]) >> 50)];
                s_ru4[lane] = Accept<T>::uniform(u52(y[2], y[3]));
                s_ru4d[lane] = u01(y[2], y[3]);
            }
            __syncthreads();
        }
        uint64_t kb64 = nsteps - s;
        if (kb64 > uint64_t(kResRngBatch - bi0)) kb64 = uint64_t(kResRngBatch - bi0);
        if (kb64 > uint64_t(kResSpec)) kb64 = kResSpec;
        if (measuring && kb64 > to_meas + 1) kb64 = to_meas + 1;   // to_meas < meas here
        const int kb = int(kb64);
        if (kb < 1) { status = GV_ERR_INVALID; break; }   // a round always resolves a step
        // this thread's terms of the kb proposals: (A^-1)(c, f) from this lane's
        // column c (one 2-column load each), u_f = phi_{2f}(t)
        cx<T> pa[kResSpec], pu[kResSpec];
        uint32_t rr[2 * kResSpec];
        int psite[kResSpec], ppart[kResSpec];   // (upf | upt << 16), (cu | cd << 16) of proposal i
        int anti = 0;   // bit i: proposal i exchanges antiparallel spins
#pragma unroll
        for (int i = 0; i < kResSpec; ++i) {
            pu[i] = cx<T>{0.f, 0.f};
            rr[2 * i] = rr[2 * i + 1] = 0u;
            psite[i] = ppart[i] = 0;
            if (i < kb) {
                const int v1 = s_rv[2 * (bi0 + i)], v2 = s_rv[2 * (bi0 + i) + 1];
                const bool up1 = s_fock[v1] >= 0, up2 = s_fock[v2] >= 0;
                if (up1 != up2) {
                    anti |= 1 << i;
                    const int upf = up1 ? v1 : v2, upt = up1 ? v2 : v1;
                    const int cu = s_fock[upf], cd = s_fock[Ns + upt];
                    psite[i] = upf | (upt << 16);
                    ppart[i] = cu | (cd << 16);
                    const int cg = g ? cd : cu;     // this flavour's particle
                    const int tg = g ? upf : upt;   // and its destination
                    uint32_t r2[2];
                    tmem_ld2(trow + 2 * cg, r2);
                    rr[2 * i] = r2[0];
                    rr[2 * i + 1] = r2[1];
                    if (f < N) {
                        const cx<T> ph = pf_bi == bi0 ? (tg == v1 ? pf[i][0] : pf[i][1]) : phase[size_t(tg) * Nk + f];
                        pu[i] = cmul_rn(ph, cf[s_sub[tg] * N + f]);
                    }
                }
            }
        }
        {   // the next round's rows, assuming it starts right after this one
            const int nb0 = bi0 + kb;
            pf_bi = -1;
            if (nb0 < kResRngBatch && s + uint64_t(kb) < nsteps) {
#pragma unroll
                for (int i = 0; i < kResSpec; ++i)
                    if (nb0 + i < kResRngBatch && s + uint64_t(kb + i) < nsteps && f < N) {
                        pf[i][0] = phase[size_t(s_rv[2 * (nb0 + i)]) * Nk + f];
                        pf[i][1] = phase[size_t(s_rv[2 * (nb0 + i) + 1]) * Nk + f];
                    }
                pf_bi = nb0;
            }
        }
        tmem_wait_ld(rr);
        T* rb = s_red + rbuf * 16 * kResSpec;
        rbuf ^= 1;
#pragma unroll
        for (int i = 0; i < kResSpec; ++i) {
            pa[i] = cx<T>{__uint_as_float(rr[2 * i]), __uint_as_float(rr[2 * i + 1])};
            if (anti & (1 << i)) {
                const cx<T> part = warp_sum(pa[i] * pu[i]);
                if (lane == 0) { rb[16 * i + warp * 2] = part.x; rb[16 * i + warp * 2 + 1] = part.y; }
            }
        }
        __syncthreads();
        int done = kb;
#pragma unroll
        for (int i = 0; i < kResSpec; ++i) {
            if (i >= kb || done < kb) continue;
            const int bi = bi0 + i;
            const int v1 = s_rv[2 * bi], v2 = s_rv[2 * bi + 1];
            int kind = 0, accepted;
            T ratio = T(1);
            if (!(anti & (1 << i))) {
                accepted = 1;   // m_weight / m_state_weight = 1 (MetroMC.cpp:41)
                ++c_noop;
            } else {
                kind = 1;
                const T* q = rb + 16 * i;
                const cx<T> ru = {q[0] + q[2] + q[4] + q[6], q[1] + q[3] + q[5] + q[7]};
                const cx<T> rd = {q[8] + q[10] + q[12] + q[14], q[9] + q[11] + q[13] + q[15]};
                ratio = Accept<T>::ratio(ru, rd);
                if (!isfinite(ratio)) { status = GV_ERR_NAN; done = -1 - i; continue; }
                accepted = ratio > T(1) ? 1 : (s_ru4[bi] < ratio);
                if (!accepted) {
                    ++c_rej;
                } else {
                    if (norm2(ru) < T(1e-9) || norm2(rd) < T(1e-9)) { status = GV_ERR_SINGULAR; done = -1 - i; continue; }
                    // occupancy of this step as read before the round's barrier
                    const int upf = psite[i] & 0xFFFF, upt = psite[i] >> 16;
                    const int dnf = upt, dnt = upf;
                    const int cu = ppart[i] & 0xFFFF, cd = ppart[i] >> 16;
                    const int cg = g ? cd : cu;
                    const cx<T> u = pu[i], a = pa[i];
                    const cx<T> ir = cinv(g ? rd : ru);
                    // w = A^-1 u: this warp's 32 rows times u_f, summed over lanes per particle
                    cx<T>* wpart = s_wpart + (g * 4 + (warp & 3)) * 128;
                    for (int c = 0; c < NCH; ++c) {
                        uint32_t r[64];
                        tmem_ld64(trow + 64 * c, r);
                        tmem_wait_ld(r);
                        cx<T> v[32];
#pragma unroll
                        for (int j = 0; j < 32; ++j) v[j] = cx<T>{__uint_as_float(r[2 * j]), __uint_as_float(r[2 * j + 1])} * u;
                        wpart[32 * c + lane] = warp_reduce_scatter(v);
                    }
                    wg_sync(g);
                    if (f < 32 * NCH) {   // w_p - [p == c]
                        const cx<T>* wp0 = s_wpart + g * 4 * 128;
                        cx<T> wq = wp0[f] + wp0[128 + f] + wp0[256 + f] + wp0[384 + f];
                        if (f == cg) wq.x -= 1.f;
                        s_w[g * 128 + f] = wq;
                    }
                    wg_sync(g);
                    // row update: AiT[f][p] -= (w_p - [p == c]) * (A^-1)(c, f) / r
                    const cx<T> coef = cneg(a * ir);
                    const cx<T>* wv = s_w + g * 128;
                    for (int c = 0; c < NCH; ++c) {
                        uint32_t r[64];
                        tmem_ld64(trow + 64 * c, r);
                        tmem_wait_ld(r);
#pragma unroll
                        for (int j = 0; j < 32; ++j) {
                            const int p = 32 * c + j;
                            cx<T> e = {__uint_as_float(r[2 * j]), __uint_as_float(r[2 * j + 1])};
                            cmac(e, wv[p], coef);
                            r[2 * j] = __float_as_uint(e.x);
                            r[2 * j + 1] = __float_as_uint(e.y);
                        }
                        tmem_st64(trow + 64 * c, r);
                    }
                    tmem_wait_st();
                    if (tid == 0) {
                        s_fock[upt] = int16_t(cu); s_fock[upf] = -1; s_part[cu] = int16_t(upt);
                        s_fock[Ns + dnt] = int16_t(cd); s_fock[Ns + dnf] = -1; s_part[N + cd] = int16_t(dnt);
                        s_racc[2 * nacc] = ru;
                        s_racc[2 * nacc + 1] = rd;
                    }
                    ++nacc;
                    ++c_acc;
                    ++since;
                    __syncthreads();
                    done = i + 1;   // the later proposals saw the old inverse and occupancy
                }
            }
            if (J.trace && w == J.trace_walker && tid == 0) {
                gv_trace t;
                t.v1 = v1; t.v2 = v2; t.kind = kind; t.accepted = accepted; t.khop = kind ? 0 : -1; t.pad = 0;
                t.ratio = double(ratio); t.u4 = s_ru4d[bi];
                J.trace[s + i] = t;
            }
        }
        if (done < 0) {   // stopped at step s - 1 - done: the walker takes no further steps
            s += uint64_t(-1 - done);
            break;
        }
        s += uint64_t(done);
        if (measuring && uint64_t(done) == to_meas + 1) {   // the round ended on a measuring step
            to_meas = meas - 1;
            if (mask & GV_MEAS_PROJHEIS) {
                // ProjHeis pass 1 from TMEM: the ratio of moving particle p of flavour g
                // to a neighbouring site j of the other flavour is
                // sum_f (A^-1)(p, f) phi_{2f}(j).  The bonds are listed by site j (the
                // four neighbours of each other-flavour particle q, entry 4 q + d), so
                // that one phase row phase[j][f] (coalesced over the lanes f) serves
                // the four bonds of j; lane f gathers (A^-1)(p, f) of each bond's
                // particle from its TMEM row (2-column loads), and each warp
                // reduce-scatters 32 bonds at a time over its lanes; the four warps'
                // partial sums meet in shared memory.
                int32_t* tab = s_nb + g * 4 * 128;   // p | kk << 8 | i << 10, or -1
                cx<T>* part_g = s_rqp + (g * 4 + (warp & 3)) * 4 * 128;
                const int NE = 4 * N;
                for (int e = f; e < NE; e += 128) {
                    const int js = s_part[(1 - g) * N + (e >> 2)];
                    const int i = s_nbr[js * 4 + (e & 3)];
                    const int pi = g ? s_fock[Ns + i] : s_fock[i];   // flavour-g particle at i, or -1
                    int kk = 0;
                    while (kk < 3 && s_nbr[i * 4 + kk] != js) ++kk;
                    tab[e] = pi >= 0 ? (pi | (kk << 8) | (i << 10)) : -1;
                }
                wg_sync(g);
                // phase rows of the eight sites of a group of 32 bonds, fetched one group ahead
                auto fetch_rows = [&](int e0, cx<T> (&ph)[8]) {
#pragma unroll
                    for (int k = 0; k < 8; ++k) {
                        const int q = (e0 >> 2) + k;
                        ph[k] = (q < N && f < N) ? phase[size_t(s_part[(1 - g) * N + q]) * Nk + f] : cx<T>{0.f, 0.f};
                    }
                };
                cx<T> phn[8];
                fetch_rows(0, phn);
                for (int e0 = 0; e0 < NE; e0 += 32) {
                    uint32_t rr[64];
                    int ent[32];
#pragma unroll
                    for (int t = 0; t < 32; ++t) {
                        ent[t] = e0 + t < NE ? tab[e0 + t] : -1;
                        uint32_t r2[2] = {0u, 0u};
                        if (ent[t] >= 0) tmem_ld2(trow + 2 * (ent[t] & 0xFF), r2);
                        rr[2 * t] = r2[0];
                        rr[2 * t + 1] = r2[1];
                    }
                    cx<T> phk[8];
#pragma unroll
                    for (int k = 0; k < 8; ++k) phk[k] = phn[k];
                    if (e0 + 32 < NE) fetch_rows(e0 + 32, phn);
#pragma unroll
                    for (int k = 0; k < 8; ++k) {   // the eight sites of this group of 32 bonds
                        const int q = (e0 >> 2) + k;
                        if (q < N && f < N) phk[k] = cmul_rn(phk[k], cf[s_sub[s_part[(1 - g) * N + q]] * N + f]);
                    }
                    tmem_wait_ld(rr);
                    cx<T> v[32];
#pragma unroll
                    for (int t = 0; t < 32; ++t)
                        v[t] = ent[t] >= 0 ? cx<T>{__uint_as_float(rr[2 * t]), __uint_as_float(rr[2 * t + 1])} * phk[t >> 2]
                                           : cx<T>{0.f, 0.f};
                    part_g[e0 + lane] = warp_reduce_scatter(v);
                }
                wg_sync(g);
                {
                    const cx<T>* q = s_rqp + g * 4 * 4 * 128;
                    for (int e = f; e < NE; e += 128) {
                        const int en = tab[e];
                        if (en >= 0) s_rq[(en >> 10) * 4 + ((en >> 8) & 3)] = q[e] + q[512 + e] + q[1024 + e] + q[1536 + e];
                    }
                }
                __syncthreads();
                projheis_from_rq<T, kResThreads>(C);
            }
            if (mask & GV_MEAS_STAGMAGN) stagmagn_now<T, kResThreads>(C);
        } else if (measuring) {
            to_meas -= uint64_t(done);
        }
    }
    k += 4 * s;
    __syncthreads();
    if (tid == 32) {
        for (int i = 0; i < nacc; ++i) {
            am = am * (to_d(s_racc[2 * i]) * to_d(s_racc[2 * i + 1]));
            amp_normalise(am, ae);
        }
    }
    // write back: both inverses from TMEM, occupancy, counters
    for (int c = 0; c < NCH; ++c) {
        uint32_t r[64];
        tmem_ld64(trow + 64 * c, r);
        tmem_wait_ld(r);
#pragma unroll
        for (int j = 0; j < 32; ++j) {
            const int p = 32 * c + j;
            if (f < N && p < N) Ag[size_t(f) * N + p] = cx<T>{__uint_as_float(r[2 * j]), __uint_as_float(r[2 * j + 1])};
        }
    }
    for (int i = tid; i < 2 * Ns; i += kResThreads) J.fock[size_t(w) * 2 * Ns + i] = s_fock[i];
    for (int i = tid; i < 2 * N; i += kResThreads) {
        const int fl = i / N, p = i % N;
        J.part[(size_t(w) * 2 + fl) * J.Nmax + p] = s_part[i];
    }
    if (tid == 0) {
        J.rng_next[w] = k;
        unsigned long long* cn = J.counts + size_t(w) * 5;
        cn[0] += c_acc + c_noop + c_rej;
        cn[1] += c_acc;
        cn[2] += c_noop;
        cn[3] += c_rej;
        J.since_reinv[w] = since;
        J.status[w] = status;
    }
    if (tid == 32) {
        J.amp_m[w] = am;
        J.amp_e[w] = ae;
    }
    tmem_fence_before();
    __syncthreads();
    tmem_fence_after();
    if (warp == 0) tmem_dealloc(tbase, kResTmemCols);
}

}  // namespace
}  // namespace gv
