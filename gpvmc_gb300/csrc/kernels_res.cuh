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
__device__ __forceinline__ void tmem_wait_ld(uint32_t (&r)[16])
{
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                   "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]),
                   "+r"(r[15])::"memory");
}
__device__ __forceinline__ void tmem_st64(uint32_t taddr, const uint32_t (&r)[64])
{
    asm volatile("tcgen05.st.sync.aligned.32x32b.x64.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32,%33,%34,%35,%36,%37,%38,%39,%40,%41,%42,%43,%44,%45,%46,%47,%48,%49,%50,%51,%52,%53,%54,%55,%56,%57,%58,%59,%60,%61,%62,%63,%64};" ::"r"(taddr), "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]), "r"(r[8]), "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15]), "r"(r[16]), "r"(r[17]), "r"(r[18]), "r"(r[19]), "r"(r[20]), "r"(r[21]), "r"(r[22]), "r"(r[23]), "r"(r[24]), "r"(r[25]), "r"(r[26]), "r"(r[27]), "r"(r[28]), "r"(r[29]), "r"(r[30]), "r"(r[31]), "r"(r[32]), "r"(r[33]), "r"(r[34]), "r"(r[35]), "r"(r[36]), "r"(r[37]), "r"(r[38]), "r"(r[39]), "r"(r[40]), "r"(r[41]), "r"(r[42]), "r"(r[43]), "r"(r[44]), "r"(r[45]), "r"(r[46]), "r"(r[47]), "r"(r[48]), "r"(r[49]), "r"(r[50]), "r"(r[51]), "r"(r[52]), "r"(r[53]), "r"(r[54]), "r"(r[55]), "r"(r[56]), "r"(r[57]), "r"(r[58]), "r"(r[59]), "r"(r[60]), "r"(r[61]), "r"(r[62]), "r"(r[63]) : "memory");
}
constexpr int kTcWaitLimit = 1 << 22;     // mbarrier polls before a wait gives up

// Poll the mbarrier phase up to `limit` times (a job's wait budget for the
// waits whose failure the kernel reports; the drain wait before TMEM is freed
// always takes the full kTcWaitLimit so that MMAs in flight finish first).
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, int limit = kTcWaitLimit)
{
    for (int i = 0; i < limit; ++i) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.b32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// ---- mbarriers and bulk (TMA) copies ----
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
// one arrival that also announces the bytes the phase's bulk copies will deliver
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
// global -> shared bulk copy completing on an mbarrier (16-byte aligned, bytes % 16 == 0)
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(dst), "l"(src), "r"(bytes), "r"(bar) : "memory");
}
// shared -> global bulk copy in this thread's bulk group
__device__ __forceinline__ void bulk_s2g(void* dst, uint32_t src, uint32_t bytes)
{
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(src), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
template <int n>
__device__ __forceinline__ void bulk_wait_read()
{
    asm volatile("cp.async.bulk.wait_group.read %0;" ::"n"(n) : "memory");
}
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
// generic-proxy shared-memory accesses of this thread before its later bulk copies
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// barrier over one warpgroup (ids 1, 2; id 0 is __syncthreads)
__device__ __forceinline__ void wg_sync(int g) { asm volatile("bar.sync %0, 128;" ::"r"(1 + g) : "memory"); }

constexpr int kResThreads = 256;
constexpr int kResTmemCols = 512;                 // both flavours, 128 complex FP32 per lane each
constexpr size_t kResMinSmem = 116 * 1024;        // over half an SM's shared memory: one CTA per SM
constexpr int kResRngBatch = 32;
constexpr int kResSpec = 8;                       // proposals evaluated per barrier (<= 32: one lane each)
constexpr int kResAccCap = 128;                   // accepted ratio pairs held before their product is taken
constexpr int kResStageRow = 34;                  // complex per staged row segment: 32 + 2 (272 B rows: no bank conflicts)

struct ResLayout {
    size_t fock, part, nbr, sub, coef, red, wpart, w, rv, ru4, ru4d, racc, rq, rqp, nb, redm, ph, bars, tbase, total, used;
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
    l.rv = al(sizeof(int16_t) * 3 * 2 * kResRngBatch);   // [batch % 3][step][v1, v2]
    l.ru4 = al(sizeof(float) * 3 * kResRngBatch);
    l.ru4d = al(sizeof(double) * 3 * kResRngBatch);
    l.racc = al(sizeof(cx<float>) * 2 * kResAccCap);     // accepted ratio pairs not yet in the amplitude
    l.rq = al(projheis ? c * 4 * Ns : 16);
    l.rqp = al(projheis ? c * 2 * 4 * 4 * 128 : 16);   // [g][warp][slot][p] partial bond ratios
    l.nb = al(projheis ? sizeof(int32_t) * 2 * 4 * 128 : 16);   // [g][bond] particle, slot and site
    l.redm = al(sizeof(double) * 4 * (kResThreads / 32));
    // phase rows of both sites of every proposal of two uniform batches
    // ([parity][step][site][N]); at launch entry and exit the same bytes hold two
    // staging tiles of the inverses ([buffer][flavour][row][kResStageRow])
    const size_t ph_rows = c * 2 * kResRngBatch * 2 * size_t(N);
    const size_t stage = c * 2 * 2 * 128 * kResStageRow;   // two buffers
    l.ph = al(ph_rows > stage ? ph_rows : stage);
    l.bars = al(sizeof(uint64_t) * 4);   // mbarriers: the two staging tiles, the two row buffers
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
    uint64_t* s_bar = reinterpret_cast<uint64_t*>(smem + lay.bars);
    const uint32_t ebar0 = smem_u32(s_bar), rbar0 = smem_u32(s_bar + 2);

    if (warp == 0) tmem_alloc(s_tbase, kResTmemCols);
    if (tid == 32) {
        for (int i = 0; i < 4; ++i) mbar_init(smem_u32(s_bar + i), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
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
    // both inverses -> TMEM (lane f = row f of AiT, zero padding), 32 particles
    // at a time: every thread copies its own row segment (256 B; N is even, so
    // 16-byte multiples) into a shared tile with one bulk (TMA) copy completing
    // on the tile's mbarrier, two segments in flight, then moves it into its
    // TMEM lane.  Every wait is bounded (J.wait_limit polls); a wait that gives
    // up ends the walker with GV_ERR_TIMEOUT after the copies in flight drained.
    cx<T>* s_stage = reinterpret_cast<cx<T>*>(smem + lay.ph);
    constexpr int kTile = 2 * 128 * kResStageRow;   // complex per staging tile
    int ne_issued = 0, ne_done = 0;                 // staging phases issued / waited for
    auto stage_segment = [&](int c) {   // particles 32c .. 32c + 31 of row f of flavour g -> tile c & 1
        const int np = N - 32 * c < 32 ? N - 32 * c : 32;
        const uint32_t bar = ebar0 + 8 * (c & 1);
        if (tid == 0) mbar_expect_tx(bar, uint32_t(2 * N) * uint32_t(np) * 8u);
        if (f < N) {
            fence_proxy_async();
            bulk_g2s(smem_u32(s_stage + (c & 1) * kTile + (g * 128 + f) * kResStageRow),
                     ai_ptr<T>(J, g, w) + size_t(f) * N + 32 * c, uint32_t(np) * 8u, bar);
        }
        ++ne_issued;
    };
    bool lost = false;   // a bounded wait gave up (block-uniform after each check)
    stage_segment(0);
    if (NCH > 1) stage_segment(1);
    for (int c = 0; c < NCH && !lost; ++c) {
        lost = !mbar_wait(ebar0 + 8 * (c & 1), (c >> 1) & 1, J.wait_limit);
        lost = __syncthreads_or(lost);   // also: every wait on this phase is over before it is armed again
        if (lost) break;
        ++ne_done;
        const cx<T>* my_seg = s_stage + (c & 1) * kTile + (g * 128 + f) * kResStageRow;
        uint32_t r[64];
#pragma unroll
        for (int j = 0; j < 16; ++j) {   // particles 32c + 2j, 32c + 2j + 1 (both < N or both >= N)
            const bool in = f < N && 32 * c + 2 * j < N;
            const float4 q = in ? reinterpret_cast<const float4*>(my_seg)[j] : make_float4(0.f, 0.f, 0.f, 0.f);
            r[4 * j] = __float_as_uint(q.x);
            r[4 * j + 1] = __float_as_uint(q.y);
            r[4 * j + 2] = __float_as_uint(q.z);
            r[4 * j + 3] = __float_as_uint(q.w);
        }
        if (c + 2 < NCH) stage_segment(c + 2);   // this thread's segment of the tile is read
        tmem_st64(trow + 64 * c, r);
    }
    tmem_wait_st();
    tmem_fence_before();
    __syncthreads();
    tmem_fence_after();
    const bool loaded = !lost;   // both inverses are in TMEM

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
    int nacc = 0;   // accepted ratio pairs waiting to be multiplied into the amplitude (block-uniform)
    // The amplitude (FP64 mantissa, base-2 exponent; LatticeStepper's running
    // product of the accepted ratios) is brought up to date only when the
    // pairs' buffer could fill within the next batch, and at the end of the
    // call: warp 1 multiplies the pending pairs as a tree (lane products, then
    // five shuffle levels, each product renormalised), so that the slow FP64
    // pipe sits on the per-step path only once every few sweeps.
    auto flush_amp = [&]() {
        if (warp == 1) {
            cx<double> v = {1.0, 0.0};
            int e = 0;
            for (int i = lane; i < nacc; i += 32) {
                v = v * (to_d(s_racc[2 * i]) * to_d(s_racc[2 * i + 1]));
                amp_normalise(v, e);
            }
#pragma unroll
            for (int o = 16; o; o >>= 1) {
                const cx<double> u = {__shfl_xor_sync(0xffffffffu, v.x, o), __shfl_xor_sync(0xffffffffu, v.y, o)};
                e += __shfl_xor_sync(0xffffffffu, e, o);
                v = v * u;
                amp_normalise(v, e);
            }
            if (lane == 0) {   // thread 32 holds the amplitude
                am = am * v;
                ae += e;
                amp_normalise(am, ae);
            }
        }
        nacc = 0;
    };
    const WalkCtx<T> C = {&J, w, Ns, N, L, Nk, N, N, s_fock, s_part, s_nbr, s_coef, s_rq, s_redm,
                          phase, ai_ptr<T>(J, 0, w), ai_ptr<T>(J, 1, w)};
    // Proposals are evaluated kResSpec at a time: every thread forms its terms
    // of the next kb proposals' ratios (same inverse, same occupancy), one
    // barrier combines them, lane i of every warp resolves proposal i, and a
    // ballot finds the first step that ends the round -- an accepted exchange,
    // whose update invalidates the later proposals (they are evaluated again,
    // from the new inverse, in the next round), or an error.  A round never
    // crosses a uniform batch or a measurement step.
    // The uniforms of a batch and the phase rows of both sites of its
    // proposals (whichever site a particle moves to, its row is there) are in
    // shared memory before the batch starts: at the start of batch b, warp 0
    // draws batch b + 2 while every warp issues bulk copies of batch b + 1's
    // rows (drawn a batch earlier), which land while batch b runs (the
    // Metropolis stream does not depend on the walk).
    cx<T>* s_ph = reinterpret_cast<cx<T>*>(smem + lay.ph);
    // warp 0: steps sb .. sb + 31 into slot rs; a step past the call's end
    // gets the sites (0, 0), so that every entry is a valid site index (the
    // FP64 uniform is kept for the trace only)
    auto draw_batch = [&](uint64_t sb, int rs) {
        int v1 = 0, v2 = 0;
        float ru = 0.f;
        double rud = 0.0;
        if (sb + lane < nsteps) {
            const uint64_t kl = k + 4 * (sb + uint64_t(lane));
            uint32_t x[4], y[4];
            philox_call(J.seed, wid, 0, kl >> 1, x);
            philox_call(J.seed, wid, 0, (kl >> 1) + 1, y);
            v1 = scaled_floor(uint32_t(Ns), u52(x[0], x[1]));
            v2 = s_nbr[v1 * 4 + int(u52(x[2], x[3]) >> 50)];
            ru = Accept<T>::uniform(u52(y[2], y[3]));
            if (J.trace) rud = u01(y[2], y[3]);
        }
        s_rv[(rs * kResRngBatch + lane) * 2] = int16_t(v1);
        s_rv[(rs * kResRngBatch + lane) * 2 + 1] = int16_t(v2);
        s_ru4[rs * kResRngBatch + lane] = ru;
        s_ru4d[rs * kResRngBatch + lane] = rud;
    };
    // all warps: the 2 x 32 phase rows of the batch in slot rs (row 2 step +
    // site, 8N bytes each) into row buffer par, one bulk copy by each of lanes
    // 0..7 of every warp, completing on that buffer's mbarrier
    static_assert(kResThreads == 256 && 2 * kResRngBatch == 64, "eight row copies per warp");
    auto fetch_batch_rows = [&](int rs, int par) {
        const uint32_t bar = rbar0 + 8 * par, rowb = uint32_t(N) * 8u;
        if (tid == 0) mbar_expect_tx(bar, uint32_t(2 * kResRngBatch) * rowb);
        if (lane < 8) {
            const int q = warp * 8 + lane;
            const int site = s_rv[(rs * kResRngBatch + (q >> 1)) * 2 + (q & 1)];
            fence_proxy_async();
            bulk_g2s(smem_u32(s_ph + (size_t(par) * 2 * kResRngBatch + q) * N), phase + size_t(site) * Nk, rowb, bar);
        }
    };
    uint32_t nb_issued = 0, nb_waited = 0;   // row batches copied / waited for
    int rs_cur = 0;                          // uniform slot of the current batch
    if (!lost) {
        if (warp == 0) {
            draw_batch(0, 0);
            draw_batch(kResRngBatch, 1);
        }
        __syncthreads();
        fetch_batch_rows(0, 0);
        nb_issued = 1;
    }
    const bool measuring = meas != 0 && mask != 0;
    // steps from s to the next measuring step (0: s itself is measured)
    uint64_t to_meas = measuring ? (meas == 1 ? 0 : (meas - (s0 % meas)) % meas) : ~uint64_t(0);
    uint64_t s = 0;
    while (!lost && s < nsteps) {
        const int bi0 = int(s % kResRngBatch);
        const int par = int(s / kResRngBatch) & 1;
        if (bi0 == 0 && s > 0) rs_cur = rs_cur == 2 ? 0 : rs_cur + 1;
        const int rs1 = rs_cur == 2 ? 0 : rs_cur + 1, rs2 = rs1 == 2 ? 0 : rs1 + 1;
        if (bi0 == 0) {
            __syncthreads();   // every thread is done with the previous batch and its buffers
            if (nacc > kResAccCap - kResRngBatch) flush_amp();   // a batch accepts at most 32
            fetch_batch_rows(rs1, par ^ 1);                              // batch b + 1's rows in flight
            if (warp == 0) draw_batch(s + 2 * kResRngBatch, rs2);        // batch b + 2's uniforms
            ++nb_issued;
            // this batch's rows (its barrier is armed again only after the next
            // batch boundary, which every thread reaches after this wait)
            const bool ok = mbar_wait(rbar0 + 8 * (nb_waited & 1), (nb_waited >> 1) & 1, J.wait_limit);
            ++nb_waited;
            if (__syncthreads_or(!ok)) { status = GV_ERR_TIMEOUT; lost = true; break; }
        }
        const int16_t* rv = s_rv + rs_cur * 2 * kResRngBatch;
        const cx<T>* prow = s_ph + size_t(par) * 2 * kResRngBatch * N;
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
        unsigned anti = 0;   // bit i: proposal i exchanges antiparallel spins
        // branch-free, so that the kResSpec chains interleave: every proposal slot
        // loads and multiplies (slots past kb, or exchanging parallel spins,
        // carry u = 0 and are ignored)
        const int fi = f < N ? f : N - 1;
#pragma unroll
        for (int i = 0; i < kResSpec; ++i) {
            const int bi = bi0 + i < kResRngBatch ? bi0 + i : kResRngBatch - 1;
            const int v1 = rv[2 * bi], v2 = rv[2 * bi + 1];
            const int u1 = s_fock[v1], u2 = s_fock[v2], d1 = s_fock[Ns + v1], d2 = s_fock[Ns + v2];
            const bool up1 = u1 >= 0, up2 = u2 >= 0;
            const bool an = i < kb && up1 != up2;
            anti |= unsigned(an) << i;
            const int upf = up1 ? v1 : v2, upt = up1 ? v2 : v1;
            const int cu = up1 ? u1 : u2, cd = up1 ? d2 : d1;   // the up particle at upf, the down one at upt
            psite[i] = upf | (upt << 16);
            ppart[i] = (cu & 0xFFFF) | (cd << 16);
            int cg = g ? cd : cu;             // this flavour's particle
            cg = cg < 0 ? 0 : cg;
            const int tg = g ? upf : upt;     // and its destination
            uint32_t r2[2];
            tmem_ld2(trow + 2 * cg, r2);
            rr[2 * i] = r2[0];
            rr[2 * i + 1] = r2[1];
            const cx<T> uu = cmul_rn(prow[size_t(2 * bi + (tg == v1 ? 0 : 1)) * N + fi], cf[s_sub[tg] * N + fi]);
            pu[i] = (an && f < N) ? uu : cx<T>{0.f, 0.f};
        }
        tmem_wait_ld(rr);
        T* rb = s_red + rbuf * 16 * kResSpec;
        rbuf ^= 1;
        {   // the kResSpec warp sums at once: a butterfly that leaves proposal
            // (lane >> 2)'s sum in lanes 4 i .. 4 i + 3 (the pairs and their order
            // are those of warp_sum, so the sums are the same)
            static_assert(kResSpec == 8, "the butterfly below sums eight proposals");
            cx<T> x[8];
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                pa[i] = cx<T>{__uint_as_float(rr[2 * i]), __uint_as_float(rr[2 * i + 1])};
                x[i] = pa[i] * pu[i];
            }
#pragma unroll
            for (int o = 16, n = 4; o >= 4; o >>= 1, n >>= 1) {
                const bool hi = (lane & o) != 0;
#pragma unroll
                for (int t = 0; t < n; ++t) {
                    const cx<T> keep = hi ? x[n + t] : x[t];
                    cx<T> send = hi ? x[t] : x[n + t];
                    send.x = __shfl_xor_sync(0xffffffffu, send.x, o);
                    send.y = __shfl_xor_sync(0xffffffffu, send.y, o);
                    x[t] = keep + send;
                }
            }
#pragma unroll
            for (int o = 2; o; o >>= 1) {
                const cx<T> y = {__shfl_xor_sync(0xffffffffu, x[0].x, o), __shfl_xor_sync(0xffffffffu, x[0].y, o)};
                x[0] = x[0] + y;
            }
            if ((lane & 3) == 0) {
                const int i = lane >> 2;
                rb[16 * i + warp * 2] = x[0].x;
                rb[16 * i + warp * 2 + 1] = x[0].y;
            }
        }
        __syncthreads();
        // lane i (i < kb) resolves proposal i; every warp does the same
        T ratio = T(1);
        int stop = 0;   // 1: accepted exchange, 2: non-finite ratio, 3: accepted with a vanishing ratio
        if (lane < kb && (anti & (1u << lane))) {
            const T* q = rb + 16 * lane;
            const cx<T> ru = {q[0] + q[2] + q[4] + q[6], q[1] + q[3] + q[5] + q[7]};
            const cx<T> rd = {q[8] + q[10] + q[12] + q[14], q[9] + q[11] + q[13] + q[15]};
            ratio = Accept<T>::ratio(ru, rd);
            if (!isfinite(ratio)) {
                stop = 2;
            } else if (ratio > T(1) || s_ru4[rs_cur * kResRngBatch + bi0 + lane] < ratio) {
                stop = (norm2(ru) < T(1e-9) || norm2(rd) < T(1e-9)) ? 3 : 1;
            }
        }
        const unsigned stops = __ballot_sync(0xffffffffu, stop != 0);
        const int first = stops ? __ffs(stops) - 1 : kb;
        const int first_kind = __shfl_sync(0xffffffffu, stop, first & 31);
        const unsigned before = (1u << first) - 1u;   // first <= kb <= kResSpec < 32
        c_noop += __popc(~anti & before);
        c_rej += __popc(anti & before);
        int done;
        if (first == kb) {
            done = kb;
        } else if (first_kind != 1) {
            status = first_kind == 2 ? GV_ERR_NAN : GV_ERR_SINGULAR;
            done = -1 - first;
        } else {
            done = first + 1;   // the later proposals saw the old inverse and occupancy
        }
        if (J.trace && w == J.trace_walker) {   // block-uniform
            const int nt = done < 0 ? -1 - done : done;
            for (int i = 0; i < nt; ++i) {
                const T ri = __shfl_sync(0xffffffffu, ratio, i);
                if (tid == 0) {
                    const int kind = (anti >> i) & 1;
                    gv_trace t;
                    t.v1 = rv[2 * (bi0 + i)]; t.v2 = rv[2 * (bi0 + i) + 1];
                    t.kind = kind; t.accepted = (!kind || i == first) ? 1 : 0; t.khop = kind ? 0 : -1; t.pad = 0;
                    t.ratio = kind ? double(ri) : 1.0; t.u4 = s_ru4d[rs_cur * kResRngBatch + bi0 + i];
                    J.trace[s + i] = t;
                }
            }
        }
        if (done > 0 && first < kb) {   // the accepted exchange of step s + first
            int ps = 0, pp = 0;
            cx<T> u = {0.f, 0.f}, a = {0.f, 0.f};
#pragma unroll
            for (int i = 0; i < kResSpec; ++i)
                if (i == first) { ps = psite[i]; pp = ppart[i]; u = pu[i]; a = pa[i]; }
            const T* q = rb + 16 * first;
            const cx<T> ru = {q[0] + q[2] + q[4] + q[6], q[1] + q[3] + q[5] + q[7]};
            const cx<T> rd = {q[8] + q[10] + q[12] + q[14], q[9] + q[11] + q[13] + q[15]};
            const int upf = ps & 0xFFFF, upt = ps >> 16;
            const int dnf = upt, dnt = upf;
            const int cu = pp & 0xFFFF, cd = pp >> 16;
            const int cg = g ? cd : cu;
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
                // phase rows of the eight sites of a group of 32 bonds and the
                // sites' coefficients, fetched one group ahead (u_f = phase * coef)
                // (branch-free: clamped indices, zeros selected afterwards)
                auto fetch_rows = [&](int e0, cx<T> (&ph)[8], cx<T> (&co)[8]) {
                    const int fi = min(f, N - 1);
                    int js[8];
#pragma unroll
                    for (int k = 0; k < 8; ++k) js[k] = s_part[(1 - g) * N + min((e0 >> 2) + k, N - 1)];
#pragma unroll
                    for (int k = 0; k < 8; ++k) {
                        ph[k] = phase[size_t(js[k]) * Nk + fi];
                        co[k] = cf[s_sub[js[k]] * N + fi];
                    }
#pragma unroll
                    for (int k = 0; k < 8; ++k)
                        if (!((e0 >> 2) + k < N && f < N)) co[k] = cx<T>{0.f, 0.f};
                };
                cx<T> phn[8], con[8];
                fetch_rows(0, phn, con);
                for (int e0 = 0; e0 < NE; e0 += 32) {
                    // the group's 32 entries first (NE is a multiple of 4: whole int4s),
                    // then the 32 TMEM loads back to back
                    int ent[32];
#pragma unroll
                    for (int q = 0; q < 8; ++q) {
                        const int4 x = e0 + 4 * q < NE ? reinterpret_cast<const int4*>(tab + e0)[q] : make_int4(-1, -1, -1, -1);
                        ent[4 * q] = x.x; ent[4 * q + 1] = x.y; ent[4 * q + 2] = x.z; ent[4 * q + 3] = x.w;
                    }
                    uint32_t rr[64];
#pragma unroll
                    for (int t = 0; t < 32; ++t) {   // branch-free: a bond without a ratio loads particle 0
                        uint32_t r2[2];
                        tmem_ld2(trow + 2 * (ent[t] >= 0 ? (ent[t] & 0xFF) : 0), r2);
                        rr[2 * t] = r2[0];
                        rr[2 * t + 1] = r2[1];
                    }
                    cx<T> phk[8];
#pragma unroll
                    for (int k = 0; k < 8; ++k) phk[k] = cmul_rn(phn[k], con[k]);   // the eight sites of this group
                    if (e0 + 32 < NE) fetch_rows(e0 + 32, phn, con);
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
    // the copies still in flight land before their bytes are used again (bounded)
    bool drained = true;
    for (; nb_waited < nb_issued; ++nb_waited)
        drained = mbar_wait(rbar0 + 8 * (nb_waited & 1), (nb_waited >> 1) & 1) && drained;
    for (; ne_done < ne_issued; ++ne_done)
        drained = mbar_wait(ebar0 + 8 * (ne_done & 1), (ne_done >> 1) & 1) && drained;
    drained = !__syncthreads_or(!drained);
    if (lost) status = GV_ERR_TIMEOUT;
    flush_amp();
    // write back (unless the inverses were not all loaded, or the tiles' bytes
    // may still be written by a copy that was not seen to land): each thread
    // moves its row segment from TMEM to its slot of a tile and stores it with
    // one bulk copy; the slot is written again two segments later, once that
    // copy has read it
    if (loaded && drained) {
        for (int c = 0; c < NCH; ++c) {
            uint32_t r[64];
            tmem_ld64(trow + 64 * c, r);
            tmem_wait_ld(r);
            if (c >= 2) bulk_wait_read<1>();
            float4* seg = reinterpret_cast<float4*>(s_stage + (c & 1) * kTile + (g * 128 + f) * kResStageRow);
#pragma unroll
            for (int j = 0; j < 16; ++j)
                seg[j] = make_float4(__uint_as_float(r[4 * j]), __uint_as_float(r[4 * j + 1]),
                                     __uint_as_float(r[4 * j + 2]), __uint_as_float(r[4 * j + 3]));
            fence_proxy_async();
            const int np = N - 32 * c < 32 ? N - 32 * c : 32;
            if (f < N) bulk_s2g(ai_ptr<T>(J, g, w) + size_t(f) * N + 32 * c, smem_u32(seg), uint32_t(np) * 8u);
            bulk_commit();
        }
        bulk_wait_all();
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
