// StatSpinStruct pair ratios on the tensor cores (mixed precision, ground
// state, N_0 = N_1 = N <= 128).  Included by engine.cu after kernels_res.cuh.
//
// StatSpinStruct (StatSpinStruct.cpp:16-135) needs, for every antiparallel
// pair (up particle c at site i, down particle q at site j), the swap ratio
//     r(c, q) = G_up(c, q) * G_dn^T(c, q),
//     G_up(c, q)   = sum_f (A_up^-1)(c, f) phi^up_f(j)   (up particle c -> site j)
//     G_dn^T(c, q) = sum_f (A_dn^-1)(q, f) phi^dn_f(i)   (down particle q -> site i)
// i.e. the G = Phi . A^-1 products of the reference's VirtUpdate for every
// pair at once.  Both are complex N x N x N matrix products per walker,
// computed here with tcgen05.mma kind::tf32 (M = 128 rows c, N = the down
// particles q rounded up to 16, K = 8 per instruction), FP32 accumulators in
// tensor memory (TMEM columns [0,128) Re G_up, [128,256) Im G_up,
// [256,384) Re G_dn^T, [384,512) Im G_dn^T; lane = row c).
//
// Split precision (Ootomo & Yokota, IJHPCA 2022): every FP32 operand x is
// split into x_hi = tf32(x) (round to nearest) and x_lo = tf32(x - x_hi);
// each real product is x_hi y_hi + x_hi y_lo + x_lo y_hi, accumulated in
// FP32, which recovers FP32 accuracy (relative error ~1e-6 per element).  A
// complex product is four real ones: Re = Ar Br + Ai (-Bi), Im = Ar Bi + Ai Br,
// the -Bi terms through the MMA's negate-B bit, so every walker and K chunk
// issues 4 x 3 x 4 = 48 MMAs per matrix.
//
// Operands are K-major in shared memory with the 128-byte swizzle: one row
// (a particle) holds 32 TF32 values of K (the Slater rows f of one chunk) in
// 128 bytes, 8-row groups 1024 bytes apart, 16-byte unit u of row r stored at
// unit u ^ (r mod 8).  The CTA's threads build the operands directly from the
// FP32 inverses (HBM) and the phase / coefficient tables (L2), so that the
// split happens on the way in; a ninth warp, which builds nothing, issues the
// MMAs from one thread and commits them to an mbarrier that the CTA waits on
// (bounded), so that the building warps fetch the next chunk meanwhile.  The
// epilogue reads the accumulators with tcgen05.ld, stages the pair ratios in
// the (then idle) tile region and adds them into the job-wide sums in
// increasing site order, so that a warp's atomics fall on a few cache lines.
// One CTA per SM (its shared memory takes more than half of the SM's),
// persistent over the walkers.
#pragma once

#include "kernels_res.cuh"

namespace gv {
namespace {

constexpr int kTcThreads = 256;          // operand-building threads (warps 0..7)
constexpr int kTcBlock = kTcThreads + 32; // + one warp that only issues the MMAs
constexpr int kTcIssuer = kTcThreads;     // its elected thread
constexpr int kTcM = 128;                 // MMA rows (up particles, zero padded)
constexpr int kOccMaxNs = 512;            // sites of the occupancy kernels and the bond lists

__host__ __device__ inline int tc_ncols(int N) { return (N + 15) & ~15; }

struct TcLayout {
    size_t a[4], b[4], site, coef, bar, tbase, red, srt, nbr, total;
};

// Operand tiles at 1024-byte multiples from a 1024-aligned base:
// A: Re hi, Re lo, Im hi, Im lo (128 rows); B: the same (tc_ncols(N) rows);
// each row 128 bytes.  The -Im terms of the complex products read the Im
// tiles through the MMA's negate-B bit.  After a walker's last MMAs the tile
// region holds its pair ratios (N x tc_ncols(N) complex FP32, at most the
// 128 KB of the tiles) for the sorted scatter into the pair sums.
__host__ __device__ inline TcLayout tc_layout(int N)
{
    TcLayout l;
    size_t o = 0;
    const size_t at = size_t(kTcM) * 128, bt = size_t(tc_ncols(N)) * 128;
    for (int i = 0; i < 4; ++i) { l.a[i] = o; o += at; }
    for (int i = 0; i < 4; ++i) { l.b[i] = o; o += bt; }
    l.site = o;
    o += sizeof(int16_t) * 2 * 2 * kTcM;     // two walkers' buffers
    l.coef = o;
    o += sizeof(cx<float>) * 2 * 4 * kTcM;
    l.bar = o;
    o += 8;
    l.tbase = o;
    o += 8;
    l.red = o;                                 // per-warp ProjHeis partial sums
    o += sizeof(double) * 4 * (kTcThreads / 32);
    l.srt = o;                                 // occupied sites in increasing order: [fl][site, particle][128], counts
    o += sizeof(int16_t) * 2 * 2 * kTcM + sizeof(int) * 2 * (kTcThreads / 32);
    l.nbr = o;                                 // neighbour table (ProjHeis mode): 4 sites per site
    o += sizeof(int16_t) * 4 * 2 * kTcM;
    l.total = o + 1024;   // room to align the base
    return l;
}

__device__ __forceinline__ uint32_t smem_addr(const void* p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Byte offset of 16-byte unit u (0..7) of row r in a K-major 128-byte-swizzled tile.
__device__ __forceinline__ uint32_t sw128(int r, int u)
{
    return uint32_t((r >> 3) * 1024 + (r & 7) * 128 + (((u ^ r) & 7) << 4));
}

// Round to the nearest TF32 value, ties away from zero, on the integer pipe:
// half a TF32 unit (bit 12) is added to the magnitude bits and the 13 bits
// below the TF32 mantissa are cleared (a carry moves into the exponent as the
// rounding requires).  For finite inputs this is the rounding of
// cvt.rna.tf32.f32, without the conversion pipe.
__device__ __forceinline__ float tf32_rna(float x)
{
    return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xFFFFE000u);
}

// Four consecutive K values of one row (real and imaginary parts) -> the
// hi / lo tiles.
__device__ __forceinline__ void tc_store_split(char* base, const size_t* tiles, uint32_t off, const float (&re)[4],
                                               const float (&im)[4])
{
    float4 rh, rl, ih, il;
    float* prh = &rh.x; float* prl = &rl.x; float* pih = &ih.x; float* pil = &il.x;
#pragma unroll
    for (int t = 0; t < 4; ++t) {
        prh[t] = tf32_rna(re[t]);
        prl[t] = tf32_rna(__fsub_rn(re[t], prh[t]));
        pih[t] = tf32_rna(im[t]);
        pil[t] = tf32_rna(__fsub_rn(im[t], pih[t]));
    }
    *reinterpret_cast<float4*>(base + tiles[0] + off) = rh;
    *reinterpret_cast<float4*>(base + tiles[1] + off) = rl;
    *reinterpret_cast<float4*>(base + tiles[2] + off) = ih;
    *reinterpret_cast<float4*>(base + tiles[3] + off) = il;
}

// Operand rows of one K chunk (f = 32 kc .. 32 kc + 31), fetched a chunk
// ahead into registers so that the global loads fly while the previous
// chunk's MMAs run.  it = threadIdx.x + 256 i numbers the (row, 16-byte unit)
// items of a tile (unit u = K values 4u .. 4u + 3).  Inverse operands (K-major
// in memory, AiT[f][r]) take row r = it % rows, unit u = it / rows: lanes run
// over rows, so a warp reads whole runs of an AiT row.  Orbital operands
// (row-major in memory, phase[site][f]) take row r = it / 8, unit u = it % 8:
// a warp reads 32 contiguous bytes of each of four phase rows.
constexpr int kTcItems = kTcM * 8 / kTcThreads;   // (row, unit) items per thread for rows <= 128

struct TcRegs {
    cx<float> inv[kTcItems][4];   // inverse operand: AiT[f][r] = (A^-1)(r, f)
    cx<float> ph[kTcItems][4];    // orbital operand: phase[site r][f]
};

// Rows r < nr of a matrix stored K-major in memory, M[f][r] at M + f ld + r rs,
// K values f < nk (zero elsewhere).
__device__ __forceinline__ void tc_load_rows(TcRegs& R, const cx<float>* M, int ld, int nr, int nk, int rows, int kc,
                                             int rs = 1)
{
#pragma unroll
    for (int i = 0; i < kTcItems; ++i) {
        const int it = threadIdx.x + kTcThreads * i, r = it % rows, u = it / rows;
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            const int f = 32 * kc + 4 * u + t;
            R.inv[i][t] = (it < rows * 8 && r < nr && f < nk) ? M[size_t(f) * ld + size_t(r) * rs] : cx<float>{0.f, 0.f};
        }
    }
}

__device__ __forceinline__ void tc_load_inverse(TcRegs& R, const cx<float>* Ai, int N, int rows, int kc)
{
    tc_load_rows(R, Ai, N, N, N, rows, kc);
}

// Phase values phase[site r][pcol[f]] of rows r < nr, K values f < nk.
__device__ __forceinline__ void tc_load_phase_cols(TcRegs& R, const cx<float>* phase, int Nk, const int16_t* site,
                                                   const int16_t* pcol, int nr, int nk, int rows, int kc)
{
#pragma unroll
    for (int i = 0; i < kTcItems; ++i) {
        const int it = threadIdx.x + kTcThreads * i, r = it >> 3, u = it & 7;
        const int s = (r < rows && r < nr) ? site[r] : -1;
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            const int f = 32 * kc + 4 * u + t;
            R.ph[i][t] = (s >= 0 && f < nk) ? phase[size_t(s) * Nk + pcol[f]] : cx<float>{0.f, 0.f};
        }
    }
}

// Phase values phase[site r][f] of rows r < N, K values f < N; four
// consecutive values as two 16-byte loads where the row stride allows.
__device__ __forceinline__ void tc_load_phase(TcRegs& R, const cx<float>* phase, int Nk, const int16_t* site, int N,
                                              int rows, int kc)
{
    const bool vec = (Nk & 1) == 0;   // 16-byte aligned pairs of complex values
#pragma unroll
    for (int i = 0; i < kTcItems; ++i) {
        const int it = threadIdx.x + kTcThreads * i, r = it >> 3, u = it & 7;
        const int s = (r < rows && r < N) ? site[r] : -1;
        const int f0 = 32 * kc + 4 * u;
        const cx<float>* p = phase + size_t(s < 0 ? 0 : s) * Nk + f0;
        if (s >= 0 && vec && f0 + 3 < N) {
            const float4 a = *reinterpret_cast<const float4*>(p);
            const float4 b = *reinterpret_cast<const float4*>(p + 2);
            R.ph[i][0] = {a.x, a.y};
            R.ph[i][1] = {a.z, a.w};
            R.ph[i][2] = {b.x, b.y};
            R.ph[i][3] = {b.z, b.w};
        } else {
#pragma unroll
            for (int t = 0; t < 4; ++t)
                R.ph[i][t] = (s >= 0 && f0 + t < N) ? p[t] : cx<float>{0.f, 0.f};
        }
    }
}

// Inverse operand rows -> split tiles.
__device__ __forceinline__ void tc_store_inverse(char* base, const size_t* tiles, const TcRegs& R, int rows)
{
#pragma unroll
    for (int i = 0; i < kTcItems; ++i) {
        const int it = threadIdx.x + kTcThreads * i;
        if (it >= rows * 8) break;
        const int r = it % rows, u = it / rows;
        float re[4], im[4];
#pragma unroll
        for (int t = 0; t < 4; ++t) { re[t] = R.inv[i][t].x; im[t] = R.inv[i][t].y; }
        tc_store_split(base, tiles, sw128(r, u), re, im);
    }
}

// Orbital operand rows phi_{2f}(site r) = phase[site][f] coef[sub(site)][f]
// (the walk's own FP32 product) -> split tiles.
__device__ __forceinline__ void tc_store_phi(char* base, const size_t* tiles, const TcRegs& R,
                                             const cx<float>* coef, const int16_t* site, int N, int L, int rows, int kc)
{
#pragma unroll
    for (int i = 0; i < kTcItems; ++i) {
        const int it = threadIdx.x + kTcThreads * i, r = it >> 3, u = it & 7;
        if (r >= rows) break;
        const int sub = r < N ? sublattice(site[r], L) : 0;
        float re[4], im[4];
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            const int f = 32 * kc + 4 * u + t;
            const cx<float> v = f < N ? cmul_rn(R.ph[i][t], coef[sub * N + f]) : cx<float>{0.f, 0.f};
            re[t] = v.x;
            im[t] = v.y;
        }
        tc_store_split(base, tiles, sw128(r, u), re, im);
    }
}

// Orbital operand with an explicit row -> coefficient table: row r, K value f
// holds phase[site r][pcol f] coef[sub(site r) * cld + f] (rows r < nr, f < nk).
__device__ __forceinline__ void tc_store_phi_cols(char* base, const size_t* tiles, const TcRegs& R,
                                                  const cx<float>* coef, int cld, const int16_t* site, int nr, int nk,
                                                  int L, int rows, int kc)
{
#pragma unroll
    for (int i = 0; i < kTcItems; ++i) {
        const int it = threadIdx.x + kTcThreads * i, r = it >> 3, u = it & 7;
        if (r >= rows) break;
        const int sub = r < nr ? sublattice(site[r], L) : 0;
        float re[4], im[4];
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            const int f = 32 * kc + 4 * u + t;
            const cx<float> v = f < nk ? cmul_rn(R.ph[i][t], coef[sub * cld + f]) : cx<float>{0.f, 0.f};
            re[t] = v.x;
            im[t] = v.y;
        }
        tc_store_split(base, tiles, sw128(r, u), re, im);
    }
}

// Shared-memory matrix descriptor: start address, leading byte offset 16
// (unused by swizzled K-major operands), stride byte offset 1024 (8-row
// groups), descriptor version 1, base offset 0, 128-byte swizzle.
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr)
{
    return uint64_t((saddr & 0x3FFFFu) >> 4) | (uint64_t(1) << 16) | (uint64_t(1024 >> 4) << 32) |
           (uint64_t(1) << 46) | (uint64_t(2) << 61);
}

// Instruction descriptor, kind::tf32: D FP32, A and B TF32, both K-major,
// no negation, N = n, M = 128.
__host__ __device__ inline uint32_t tc_idesc(int n)
{
    return (1u << 4) | (2u << 7) | (2u << 10) | (uint32_t(n >> 3) << 17) | (uint32_t(kTcM >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void tc_commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}


__device__ __forceinline__ void tmem_wait_ld(uint32_t (&r)[32])
{
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                   "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]), "+r"(r[15]),
                   "+r"(r[16]), "+r"(r[17]), "+r"(r[18]), "+r"(r[19]), "+r"(r[20]), "+r"(r[21]), "+r"(r[22]), "+r"(r[23]),
                   "+r"(r[24]), "+r"(r[25]), "+r"(r[26]), "+r"(r[27]), "+r"(r[28]), "+r"(r[29]), "+r"(r[30]), "+r"(r[31])::"memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t* r)
{
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                 : "r"(taddr));
}

// The 48 MMAs of one K chunk into the accumulator pair at column dcol:
// Re += Ar Br + Ai (-Bi), Im += Ar Bi + Ai Br, each real product as three
// split-precision terms, K = 8 per instruction (32 bytes along the row).
// The -Bi terms read the Bi tiles through the instruction descriptor's
// negate-B bit (bit 14).
__device__ __forceinline__ void tc_issue_chunk(uint32_t tbase, uint32_t dcol, uint32_t sbase, const TcLayout& lay,
                                               uint32_t idesc, bool first)
{
    enum { RH = 0, RL = 1, IH = 2, IL = 3 };
    const int re_terms[6][2] = {{RH, RH}, {RH, RL}, {RL, RH}, {IH, IH}, {IH, IL}, {IL, IH}};
    const uint32_t idesc_neg = idesc | (1u << 14);
    const int im_terms[6][2] = {{RH, IH}, {RH, IL}, {RL, IH}, {IH, RH}, {IH, RL}, {IL, RH}};
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) {
#pragma unroll
        for (int t = 0; t < 6; ++t) {
            const uint32_t acc = (first && kk == 0 && t == 0) ? 0u : 1u;
            tc_mma(tbase + dcol, tc_desc(sbase + uint32_t(lay.a[re_terms[t][0]]) + 32 * kk),
                   tc_desc(sbase + uint32_t(lay.b[re_terms[t][1]]) + 32 * kk), t >= 3 ? idesc_neg : idesc, acc);
            tc_mma(tbase + dcol + 128, tc_desc(sbase + uint32_t(lay.a[im_terms[t][0]]) + 32 * kk),
                   tc_desc(sbase + uint32_t(lay.b[im_terms[t][1]]) + 32 * kk), idesc, acc);
        }
    }
}

// The job-wide pair sums (StatSpinStruct m_vals in compact form):
//   T[i][j]   += r  for up site i, down site j (complex),
//   Aud[i][j] += 1  (antiparallel count, from k_occ_pairs),
// from which szz, s+- and s-+ follow (gv_job_read_statspin).
//
// Work of one CTA: its walkers w = blockIdx.x + k gridDim.x in turn, each as
// 2 KC chunks (G_up then G_dn^T, KC = ceil(N / 32) K chunks each).  Per chunk:
// wait for the previous chunk's MMAs (the tiles are free), split the
// prefetched operand rows into the tiles, issue 48 MMAs and commit them, then
// fetch the next chunk's rows (the next walker's first chunk after the last
// one) while the MMAs run.  The epilogue of a walker follows its last chunk;
// the per-walker tables (sites, coefficients) are double-buffered so that the
// next walker's first rows can be fetched before it.
// The walkers after w that a CTA gives up before reaching (a bounded wait ran
// out on walker w): marked GV_ERR_TIMEOUT as well, so that no later kernel of
// the measurement reads results that were never written.  Called by one thread.
__device__ __forceinline__ void tc_mark_rest(const DevJob& J, int w)
{
    for (int r = w + int(gridDim.x); r < J.W; r += gridDim.x)
        if (J.status[r] == GV_OK) J.status[r] = GV_ERR_TIMEOUT;
}

__device__ __forceinline__ int tc_next_walker(const DevJob& J, int w)
{
    for (w += gridDim.x; w < J.W; w += gridDim.x)
        if (J.status[w] == GV_OK) return w;
    return -1;
}

// The FP32 staging sums of one StatSpinStruct measurement (vector atomics of
// k_statspin_tc) into the FP64 job-wide sums T, and back to zero.
__global__ void k_fold_ss(DevJob J)
{
    const size_t n = size_t(J.Ns) * J.Ns;
    for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
        const float2 v = J.ss32[i];
        if (v.x != 0.f || v.y != 0.f) {
            J.ss[2 * i] += f32_to_f64(v.x);
            J.ss[2 * i + 1] += f32_to_f64(v.y);
            J.ss32[i] = make_float2(0.f, 0.f);
        }
    }
}

// mode bit 0: StatSpinStruct pair sums (StatSpinStruct.cpp:16-135); bit 1:
// ProjHeis (ProjHeis.cpp:40-158) from the same products: the pairs whose up
// and down sites are nearest neighbours are the antiparallel bonds, and with
// n_anti of them E/site = (Ns / 2 - n_anti / 2 - sum_bonds r / 2) / Ns per
// walker (parallel bonds +1/4, antiparallel -1/4 - r/2).
__global__ void __launch_bounds__(kTcBlock, 1) k_statspin_tc(DevJob J, int mode)
{
    extern __shared__ __align__(16) char smem_raw[];
    const uint32_t raw = smem_addr(smem_raw);
    char* base = smem_raw + ((1024u - (raw & 1023u)) & 1023u);
    const uint32_t sbase = smem_addr(base);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int N = J.N[0], Nt = tc_ncols(N), Ns = J.Ns, L = J.L, Nk = J.Nk;
    const TcLayout lay = tc_layout(N);
    int16_t* s_site = reinterpret_cast<int16_t*>(base + lay.site);      // [buf][fl][p]
    cx<float>* s_coef = reinterpret_cast<cx<float>*>(base + lay.coef);  // [buf][fl][sub][f]
    uint64_t* s_bar = reinterpret_cast<uint64_t*>(base + lay.bar);
    uint32_t* s_tbase = reinterpret_cast<uint32_t*>(base + lay.tbase);
    double* s_red = reinterpret_cast<double*>(base + lay.red);
    const uint32_t bar = smem_addr(s_bar);

    if (warp == 0) tmem_alloc(s_tbase, 512);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    tmem_fence_before();
    __syncthreads();
    tmem_fence_after();
    const uint32_t tbase = *s_tbase;
    const uint32_t idesc = tc_idesc(Nt);
    const int KC = (N + 31) / 32;
    uint32_t parity = 0;
    bool failed = false;

    const bool worker = tid < kTcThreads;   // the issuing warp builds no operands
    int16_t* s_nbr = reinterpret_cast<int16_t*>(base + lay.nbr);      // [site][4]
    if (mode & 2)
        for (int i = tid; i < 4 * Ns; i += kTcBlock) s_nbr[i] = int16_t(J.nbr[i]);   // read after the barriers below

    // per-walker tables into buffer b
    auto tables = [&](int w, int b) {
        if (!worker) return;
        int16_t* st = s_site + b * 2 * kTcM;
        cx<float>* sc = s_coef + b * 4 * kTcM;
        for (int i = tid; i < 2 * N; i += kTcThreads) {
            const int fl = i / N, p = i % N;
            st[fl * kTcM + p] = J.part[(size_t(w) * 2 + fl) * J.Nmax + p];
        }
        const cx<float>* cg = J.coef32 + size_t(w) * 4 * Ns;   // [fl][sub][orbital]
        for (int i = tid; i < 4 * N; i += kTcThreads) {
            const int fl = i / (2 * N), sub = (i / N) & 1, f = i % N;
            sc[i] = cg[(size_t(fl) * 2 + sub) * Ns + 2 * f];
        }
    };
    // chunk (gm, kc) of walker w: the inverse operand is A for G_up and B for
    // G_dn^T; the orbital operand the other one
    auto fetch = [&](TcRegs& R, int w, int b, int gm, int kc) {
        if (!worker) return;
        const int16_t* st = s_site + b * 2 * kTcM;
        tc_load_inverse(R, ai_ptr<float>(J, gm, w), N, gm == 0 ? kTcM : Nt, kc);
        tc_load_phase(R, J.phase32, Nk, gm == 0 ? st + kTcM : st, N, gm == 0 ? Nt : kTcM, kc);
    };

    int w = blockIdx.x < J.W ? int(blockIdx.x) : -1;
    if (w >= 0 && J.status[w] != GV_OK) w = tc_next_walker(J, w);
    TcRegs R;
    int b = 0;
    if (w >= 0) {
        tables(w, 0);
        __syncthreads();
        fetch(R, w, 0, 0, 0);
    }
    bool first = true;   // no MMAs of this walker in flight yet
    while (w >= 0 && !failed) {
        const int wn = tc_next_walker(J, w);
        const int16_t* st = s_site + b * 2 * kTcM;
        const cx<float>* sc = s_coef + b * 4 * kTcM;
        // site lists of the walker for the epilogue: fk = particle at site tid
        // of each flavour (or -1), loaded at step 0; occ = the warp's ballot
        // of the sites that list a particle, counted per warp at step 1
        int16_t* srt = reinterpret_cast<int16_t*>(base + lay.srt);   // [fl][site | particle][kTcM]
        int* s_cnt = reinterpret_cast<int*>(srt + 4 * kTcM);          // [warp][fl]
        int fk[2] = {-1, -1};
        unsigned occ[2] = {0u, 0u};
        int qn[4] = {-1, -1, -1, -1};   // ProjHeis only: down particle at each neighbour of row c's site, or -1
        for (int step = 0; step < 2 * KC; ++step) {
            const int gm = step / KC, kc = step % KC;
            if (!first) {   // the previous chunk's MMAs are done with the tiles
                const bool ok = mbar_wait(bar, parity, J.wait_limit);
                if (__syncthreads_or(!ok)) { failed = true; break; }
                parity ^= 1u;
            }
            first = false;
            if (!worker) {
            } else if (gm == 0) {   // G_up: A = AiT_up^T (rows c), B = Phi_up at the down sites (rows q)
                tc_store_inverse(base, lay.a, R, kTcM);
                tc_store_phi(base, lay.b, R, sc, st + kTcM, N, L, Nt, kc);
            } else {                // G_dn^T: A = Phi_dn at the up sites (rows c), B = AiT_dn^T (rows q)
                tc_store_phi(base, lay.a, R, sc + 2 * N, st, N, L, kTcM, kc);
                tc_store_inverse(base, lay.b, R, Nt);
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            tmem_fence_before();
            __syncthreads();
            if (tid == kTcIssuer) {   // the building warps go on to fetch the next chunk meanwhile
                tmem_fence_after();
                tc_issue_chunk(tbase, uint32_t(256 * gm), sbase, lay, idesc, kc == 0);
                tc_commit(bar);
            }
            if (step + 1 < 2 * KC) {
                fetch(R, w, b, (step + 1) / KC, (step + 1) % KC);
            } else if (wn >= 0) {
                tables(wn, b ^ 1);
                __syncthreads();
                fetch(R, wn, b ^ 1, 0, 0);
            }
            if (step == 0 && worker && tid < Ns) {   // loads that land while the MMAs run
                fk[0] = J.fock[size_t(w) * 2 * Ns + tid];
                fk[1] = J.fock[(size_t(w) * 2 + 1) * Ns + tid];
            }
            if (step == 0 && worker && mode == 2) {   // ProjHeis only: the down particles next to row c's site
                const int c = 32 * (warp & 3) + lane;
                const int si = c < N ? st[c] : -1;
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const int v = si >= 0 ? s_nbr[si * 4 + k] : -1;
                    bool dup = false;
#pragma unroll
                    for (int k2 = 0; k2 < k; ++k2) dup = dup || (si >= 0 && s_nbr[si * 4 + k2] == v);
                    qn[k] = (v >= 0 && !dup) ? J.fock[(size_t(w) * 2 + 1) * Ns + v] : -1;
                }
            }
            if (step == 1 && worker) {   // only particle indices that address V are listed
                occ[0] = __ballot_sync(0xffffffffu, fk[0] >= 0 && fk[0] < N);
                occ[1] = __ballot_sync(0xffffffffu, fk[1] >= 0 && fk[1] < N);
                if (lane == 0) { s_cnt[warp * 2] = __popc(occ[0]); s_cnt[warp * 2 + 1] = __popc(occ[1]); }
            }
        }
        if (failed) {
            if (tid == 0) J.status[w] = GV_ERR_TIMEOUT;
            break;
        }
        {
            const bool ok = mbar_wait(bar, parity, J.wait_limit);
            if (__syncthreads_or(!ok)) {
                failed = true;
                if (tid == 0) J.status[w] = GV_ERR_TIMEOUT;
                break;
            }
            parity ^= 1u;
        }
        tmem_fence_after();
        cx<double> eb = {0.0, 0.0};   // sum of the bond ratios of this thread's pairs
        int nanti = 0;
        if (mode != 2) {   // StatSpinStruct (and ProjHeis from the same pairs)
            // epilogue.  (1) the sorted site lists: site and particle of the k-th
            // occupied site of each flavour (the per-warp counts were written at
            // step 1, before the barriers since)
            if (worker) {
                const unsigned below = (1u << lane) - 1u;
    #pragma unroll
                for (int fl = 0; fl < 2; ++fl) {
                    if ((occ[fl] >> lane) & 1u) {
                        int off = __popc(occ[fl] & below);
                        for (int q = 0; q < warp; ++q) off += s_cnt[q * 2 + fl];
                        if (off < kTcM) {
                            srt[fl * 2 * kTcM + off] = int16_t(tid);
                            srt[fl * 2 * kTcM + kTcM + off] = int16_t(fk[fl]);
                        }
                    }
                }
            }
            // (2) warp -> TMEM lanes 32 (warp % 4) .. +31 (rows c), 16-column chunks
            // of q split between the two warps of a lane group; the pair ratios
            // r(c, q) go to V in the tile region, row c, the pairs (q, q + 1) of
            // even q at pair slot (q / 2) ^ (c % 8) (the XOR spreads a column's
            // rows over the banks; a pair is one 16-byte store)
            cx<float>* V = reinterpret_cast<cx<float>*>(base);
            {
                const int lg = warp & 3, c = 32 * lg + lane;
                for (int cc = warp >> 2; worker && cc < Nt / 16; cc += 2) {
                    uint32_t r[64];
                    const uint32_t ta = tbase + (uint32_t(32 * lg) << 16) + uint32_t(16 * cc);
                    tmem_ld16(ta, r);
                    tmem_ld16(ta + 128, r + 16);
                    tmem_ld16(ta + 256, r + 32);
                    tmem_ld16(ta + 384, r + 48);
                    tmem_wait_ld(r);
                    if (c < N) {
    #pragma unroll
                        for (int t = 0; t < 16; t += 2) {
                            const cx<float> v0 = cmul_rn(cx<float>{__uint_as_float(r[t]), __uint_as_float(r[16 + t])},
                                                         cx<float>{__uint_as_float(r[32 + t]), __uint_as_float(r[48 + t])});
                            const cx<float> v1 =
                                cmul_rn(cx<float>{__uint_as_float(r[t + 1]), __uint_as_float(r[17 + t])},
                                        cx<float>{__uint_as_float(r[33 + t]), __uint_as_float(r[49 + t])});
                            const int slot = ((16 * cc + t) >> 1) ^ (c & 7);
                            *reinterpret_cast<float4*>(V + c * Nt + 2 * slot) = make_float4(v0.x, v0.y, v1.x, v1.y);
                        }
                    }
                }
            }
            tmem_fence_before();
            __syncthreads();
            // (4) pair sums in site order: warp -> up sites a = warp, warp + 8, ...;
            // lane -> down sites b = lane + 32 k, so that one atomic instruction
            // covers 32 increasing sites of one row of the table
            if (worker) {
                const int16_t* ups = srt;
                const int16_t* upp = srt + kTcM;
                const int16_t* dns = srt + 2 * kTcM;
                const int16_t* dnp = srt + 3 * kTcM;
                int n_up = 0, n_dn = 0;   // entries written for this walker (N each for a consistent state)
                for (int q = 0; q < kTcThreads / 32; ++q) { n_up += s_cnt[q * 2]; n_dn += s_cnt[q * 2 + 1]; }
                n_up = min(n_up, kTcM);
                n_dn = min(n_dn, kTcM);
                int jj[kTcM / 32], qq[kTcM / 32];
    #pragma unroll
                for (int k = 0; k < kTcM / 32; ++k) {
                    const int bq = lane + 32 * k;
                    jj[k] = bq < n_dn ? dns[bq] : -1;
                    qq[k] = bq < n_dn ? dnp[bq] : 0;
                }
                for (int a = warp; a < n_up; a += kTcThreads / 32) {
                    const int i = ups[a], c = upp[a];
                    const cx<float>* Vc = V + c * Nt;
                    const int sw = c & 7;
                    float2* Ti = J.ss32 + size_t(i) * Ns;
                    int nb[4] = {-1, -1, -1, -1};
                    if (mode & 2) {
    #pragma unroll
                        for (int k = 0; k < 4; ++k) nb[k] = s_nbr[i * 4 + k];
                    }
    #pragma unroll
                    for (int k = 0; k < kTcM / 32; ++k) {
                        if (jj[k] < 0) continue;
                        const cx<float> v = Vc[2 * ((qq[k] >> 1) ^ sw) + (qq[k] & 1)];
                        if (mode & 1)   // FP32 staging sums, folded into the FP64 sums after the launch
                            atomicAdd(Ti + jj[k], make_float2(v.x, v.y));
                        if ((mode & 2) && (jj[k] == nb[0] || jj[k] == nb[1] || jj[k] == nb[2] || jj[k] == nb[3])) {
                            eb.x += f32_to_f64(v.x);
                            eb.y += f32_to_f64(v.y);
                            ++nanti;
                        }
                    }
                }
            }
        } else {
            // ProjHeis only: the thread of row c takes its up particle's
            // antiparallel bonds (columns qn) straight out of the TMEM loads
            const int lg = warp & 3, c = 32 * lg + lane;
            for (int cc = warp >> 2; worker && cc < Nt / 16; cc += 2) {
                uint32_t r[64];
                const uint32_t ta = tbase + (uint32_t(32 * lg) << 16) + uint32_t(16 * cc);
                tmem_ld16(ta, r);
                tmem_ld16(ta + 128, r + 16);
                tmem_ld16(ta + 256, r + 32);
                tmem_ld16(ta + 384, r + 48);
                tmem_wait_ld(r);
                if (c < N) {
#pragma unroll
                    for (int t = 0; t < 16; ++t) {
                        const int q = 16 * cc + t;
                        if (q == qn[0] || q == qn[1] || q == qn[2] || q == qn[3]) {
                            const cx<float> v =
                                cmul_rn(cx<float>{__uint_as_float(r[t]), __uint_as_float(r[16 + t])},
                                        cx<float>{__uint_as_float(r[32 + t]), __uint_as_float(r[48 + t])});
                            eb.x += f32_to_f64(v.x);
                            eb.y += f32_to_f64(v.y);
                            ++nanti;
                        }
                    }
                }
            }
            tmem_fence_before();
        }
        if (mode & 2) {   // the walker's ProjHeis sample
#pragma unroll
            for (int o = 16; o; o >>= 1) {
                eb.x += __shfl_xor_sync(0xffffffffu, eb.x, o);
                eb.y += __shfl_xor_sync(0xffffffffu, eb.y, o);
                nanti += __shfl_xor_sync(0xffffffffu, nanti, o);
            }
            if (lane == 0 && worker) { s_red[warp * 4] = eb.x; s_red[warp * 4 + 1] = eb.y; s_red[warp * 4 + 2] = double(nanti); }
            __syncthreads();
            if (tid == 0) {
                double ex = 0.0, ey = 0.0, na = 0.0;
                for (int q = 0; q < kTcThreads / 32; ++q) { ex += s_red[q * 4]; ey += s_red[q * 4 + 1]; na += s_red[q * 4 + 2]; }
                const double inv_ns = 1.0 / double(Ns);
                J.pj[size_t(w) * 2].x += (0.5 * Ns - 0.5 * na - 0.5 * ex) * inv_ns;
                J.pj[size_t(w) * 2].y += -0.5 * ey * inv_ns;
                J.pj[size_t(w) * 2 + 1].x += 1.0;
                J.pj_n[w] += 1;
            }
        }
        if (tid == 0 && (mode & 1)) atomicAdd(J.ss_n, w == 0 ? 1 : 0);
        __syncthreads();   // V is read: the next walker's operands may overwrite the tiles
        first = true;   // the next walker's first MMAs follow the __syncthreads of its first chunk
        w = wn;
        b ^= 1;
    }
    if (failed && tid == 0) tc_mark_rest(J, w);
    if (failed) mbar_wait(bar, parity);   // the phase that timed out: MMAs in flight finish before TMEM is freed
    tmem_fence_before();
    __syncthreads();
    tmem_fence_after();
    if (warp == 0) tmem_dealloc(tbase, 512);
}

// ---- Exciton overlap rows on the tensor cores (mixed exciton channel) ----
// The exciton ProjHeis needs, for every channel state k and every flavour-1
// site d, Z[k][d] = sum_f GupT[f][k] phi_{worb0[f]}(d) (the R A^-1 C block of
// linalg::DetUpdate for all states and all bond targets at once,
// linalg.cpp:274-290): per walker an Nexc x N0 x N1 complex product.  Same
// split-TF32 scheme and pipeline as k_statspin_tc: A = GupT^T (rows k, K = f),
// B = Phi_0 at the flavour-1 sites (rows d), one accumulator pair in TMEM
// (256 columns).  Output Z[w][d][k] (FP32, k fastest) for k_measure_trans.
constexpr int kTcMaxK = 160;   // N0 <= 160 (five K chunks)

__host__ __device__ inline TcLayout tc_layout_z(int N1)
{
    TcLayout l;
    size_t o = 0;
    const size_t at = size_t(kTcM) * 128, bt = size_t(tc_ncols(N1)) * 128;
    for (int i = 0; i < 4; ++i) { l.a[i] = o; o += at; }
    for (int i = 0; i < 4; ++i) { l.b[i] = o; o += bt; }
    l.site = o;   // [buf][ flavour-1 sites (128) | phase column of row f (kTcMaxK) ]
    o += sizeof(int16_t) * 2 * (kTcM + kTcMaxK);
    l.coef = o;   // [buf][sub][f]
    o += sizeof(cx<float>) * 2 * 2 * kTcMaxK;
    l.bar = o;
    o += 8;
    l.tbase = o;
    o += 8;
    l.total = o + 1024;
    return l;
}

__global__ void __launch_bounds__(kTcBlock, 1) k_trans_z_tc(DevJob J, cx<float>* Z)
{
    extern __shared__ __align__(16) char smem_raw[];
    const uint32_t raw = smem_addr(smem_raw);
    char* base = smem_raw + ((1024u - (raw & 1023u)) & 1023u);
    const uint32_t sbase = smem_addr(base);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int N0 = J.N[0], N1 = J.N[1], Nexc = J.Nexc, Nt = tc_ncols(N1), Ns = J.Ns, L = J.L, Nk = J.Nk;
    const TcLayout lay = tc_layout_z(N1);
    int16_t* s_tab = reinterpret_cast<int16_t*>(base + lay.site);
    cx<float>* s_cf = reinterpret_cast<cx<float>*>(base + lay.coef);
    uint64_t* s_bar = reinterpret_cast<uint64_t*>(base + lay.bar);
    uint32_t* s_tbase = reinterpret_cast<uint32_t*>(base + lay.tbase);
    const uint32_t bar = smem_addr(s_bar);

    if (warp == 0) tmem_alloc(s_tbase, 256);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    tmem_fence_before();
    __syncthreads();
    tmem_fence_after();
    const uint32_t tbase = *s_tbase;
    const uint32_t idesc = tc_idesc(Nt);
    const int KC = (N0 + 31) / 32;
    uint32_t parity = 0;
    bool failed = false;

    const bool worker = tid < kTcThreads;   // the issuing warp builds no operands
    auto tables = [&](int w, int b) {
        if (!worker) return;
        int16_t* site = s_tab + b * (kTcM + kTcMaxK);
        int16_t* pcol = site + kTcM;
        cx<float>* cf = s_cf + b * 2 * kTcMaxK;
        for (int d = tid; d < N1; d += kTcThreads) site[d] = J.part[(size_t(w) * 2 + 1) * J.Nmax + d];
        const cx<float>* cg = J.coef32 + size_t(w) * 4 * Ns;   // flavour 0: [sub][orbital]
        for (int i = tid; i < 2 * N0; i += kTcThreads) {
            const int sub = i / N0, f = i % N0;
            const int o = J.worb[size_t(w) * 2 * J.Nmax + f];
            cf[sub * kTcMaxK + f] = cg[size_t(sub) * Ns + o];
            if (!sub) pcol[f] = int16_t(o >> 1);
        }
    };
    auto fetch = [&](TcRegs& R, int w, int b, int kc) {
        if (!worker) return;
        const int16_t* site = s_tab + b * (kTcM + kTcMaxK);
        const cx<float>* G = static_cast<const cx<float>*>(J.gup) + size_t(w) * N0 * Nexc;
        tc_load_rows(R, G, Nexc, Nexc, N0, kTcM, kc);
        tc_load_phase_cols(R, J.phase32, Nk, site, site + kTcM, N1, N0, Nt, kc);
    };

    int w = blockIdx.x < J.W ? int(blockIdx.x) : -1;
    if (w >= 0 && J.status[w] != GV_OK) w = tc_next_walker(J, w);
    TcRegs R;
    int b = 0;
    if (w >= 0) {
        tables(w, 0);
        __syncthreads();
        fetch(R, w, 0, 0);
    }
    bool first = true;
    while (w >= 0 && !failed) {
        const int wn = tc_next_walker(J, w);
        const int16_t* site = s_tab + b * (kTcM + kTcMaxK);
        const cx<float>* cf = s_cf + b * 2 * kTcMaxK;
        for (int kc = 0; kc < KC; ++kc) {
            if (!first) {
                const bool ok = mbar_wait(bar, parity, J.wait_limit);
                if (__syncthreads_or(!ok)) { failed = true; break; }
                parity ^= 1u;
            }
            first = false;
            if (worker) {
                tc_store_inverse(base, lay.a, R, kTcM);
                tc_store_phi_cols(base, lay.b, R, cf, kTcMaxK, site, N1, N0, L, Nt, kc);
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            tmem_fence_before();
            __syncthreads();
            if (tid == kTcIssuer) {
                tmem_fence_after();
                tc_issue_chunk(tbase, 0u, sbase, lay, idesc, kc == 0);
                tc_commit(bar);
            }
            if (kc + 1 < KC) {
                fetch(R, w, b, kc + 1);
            } else if (wn >= 0) {
                tables(wn, b ^ 1);
                __syncthreads();
                fetch(R, wn, b ^ 1, 0);
            }
        }
        if (failed) {
            if (tid == 0) J.status[w] = GV_ERR_TIMEOUT;
            break;
        }
        {
            const bool ok = mbar_wait(bar, parity, J.wait_limit);
            if (__syncthreads_or(!ok)) {
                failed = true;
                if (tid == 0) J.status[w] = GV_ERR_TIMEOUT;
                break;
            }
            parity ^= 1u;
        }
        tmem_fence_after();
        // epilogue: lane k of TMEM -> Z[w][d][k], 16 columns d at a time
        const int lg = warp & 3, k = 32 * lg + lane;
        for (int cc = warp >> 2; worker && cc < Nt / 16; cc += 2) {
            uint32_t r[32];
            const uint32_t ta = tbase + (uint32_t(32 * lg) << 16) + uint32_t(16 * cc);
            tmem_ld16(ta, r);
            tmem_ld16(ta + 128, r + 16);
            tmem_wait_ld(r);
            if (k < Nexc) {
#pragma unroll
                for (int t = 0; t < 16; ++t) {
                    const int d = 16 * cc + t;
                    if (d < N1)
                        Z[(size_t(w) * N1 + d) * Nexc + k] = cx<float>{__uint_as_float(r[t]), __uint_as_float(r[16 + t])};
                }
            }
        }
        tmem_fence_before();
        first = true;
        w = wn;
        b ^= 1;
    }
    if (failed && tid == 0) tc_mark_rest(J, w);
    if (failed) mbar_wait(bar, parity);
    tmem_fence_before();
    __syncthreads();
    tmem_fence_after();
    if (warp == 0) tmem_dealloc(tbase, 256);
}

// ---- Longitudinal-exciton overlap sums on the tensor cores (mixed) ----
// The longitudinal ProjHeis needs, for every antiparallel bond b (flavour 0
// moving s0 -> t0, flavour 1 t0 -> s0) and every orbital o of each flavour,
//     Z_b[fl][o] = sum_f R_fl[f][o] C_b,fl[f],   C_b,fl[f] = phi_{worb_fl[f]}(t_b,fl)
// (t_b,0 = t0, t_b,1 = s0): the Z_o of linalg::DetUpdate's capacitance
// matrices (linalg.cpp:107-400) for all bonds at once, per walker and flavour
// an (Ns/2 x N) x (N x nanti) complex product over the upper-band orbitals
// o = 2 r + 1, the orbitals the channel states enter (their Z is all the
// measurement reads, apart from the current hole's, which it forms itself).
// Same split-TF32 scheme and pipeline as k_trans_z_tc: A = R_fl^T (rows o,
// 128 per tile, K = f), B = the bonds' new columns (rows b, 128 per chunk),
// one accumulator pair in TMEM (256 columns, lane = o).  The bonds are listed
// in creation order (SquareLattice.cpp:9-28), as k_measure_long lists them.
// Output Z[w][fl][b][r] (FP32, the odd orbitals o = 2 r + 1 fastest, b < 2 Ns)
// for k_measure_long.
__host__ __device__ inline TcLayout tc_layout_lz(int N)
{
    TcLayout l;
    size_t o = 0;
    const size_t t = size_t(kTcM) * 128;
    for (int i = 0; i < 4; ++i) { l.a[i] = o; o += t; }
    for (int i = 0; i < 4; ++i) { l.b[i] = o; o += t; }
    l.site = o;   // [fl][bond] new site of the flavour's moving particle, then [fl][f] phase column of row f
    o += sizeof(int16_t) * 2 * (2 * kOccMaxNs + kTcM);
    l.coef = o;   // [fl][sub][f] coefficient of row f's orbital
    o += sizeof(cx<float>) * 2 * 2 * kTcM;
    l.bar = o;
    o += 8;
    l.tbase = o;
    o += 8;
    l.red = o;    // per-warp bond counts
    o += sizeof(int) * (kTcBlock / 32 + 1);
    l.srt = l.nbr = 0;
    l.total = o + 1024;
    (void)N;
    return l;
}

__global__ void __launch_bounds__(kTcBlock, 1) k_long_z_tc(DevJob J, cx<float>* Z)
{
    extern __shared__ __align__(16) char smem_raw[];
    const uint32_t raw = smem_addr(smem_raw);
    char* base = smem_raw + ((1024u - (raw & 1023u)) & 1023u);
    const uint32_t sbase = smem_addr(base);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int N = J.N[0], Ns = J.Ns, L = J.L, Nk = J.Nk, Nmax = J.Nmax, Bmax = 2 * Ns;
    const TcLayout lay = tc_layout_lz(N);
    int16_t* s_bs = reinterpret_cast<int16_t*>(base + lay.site);   // [fl][b]
    int16_t* s_pcol = s_bs + 2 * 2 * kOccMaxNs;                     // [fl][f]
    cx<float>* s_cf = reinterpret_cast<cx<float>*>(base + lay.coef);   // [fl][sub][f]
    uint64_t* s_bar = reinterpret_cast<uint64_t*>(base + lay.bar);
    uint32_t* s_tbase = reinterpret_cast<uint32_t*>(base + lay.tbase);
    int* s_cnt = reinterpret_cast<int*>(base + lay.red);
    const uint32_t bar = smem_addr(s_bar);

    if (warp == 0) tmem_alloc(s_tbase, 256);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    tmem_fence_before();
    __syncthreads();
    tmem_fence_after();
    const uint32_t tbase = *s_tbase;
    const uint32_t idesc = tc_idesc(kTcM);
    const int KC = (N + 31) / 32;
    const int No = Ns / 2;                   // upper-band (odd) orbitals
    const int MT = (No + kTcM - 1) / kTcM;   // orbital tiles
    uint32_t parity = 0;
    bool failed = false;
    const bool worker = tid < kTcThreads;   // the issuing warp builds no operands
    int nanti = 0;

    // the walker's bond list (all threads; ends synchronised) and row tables
    auto tables = [&](int w) {
        nanti = 0;
        for (int e0 = 0; e0 < Bmax; e0 += kTcBlock) {
            const int e = e0 + tid;
            bool anti = false;
            int s0 = 0, t0 = 0;
            if (e < Bmax) {
                const int4 E = J.edges[e];
                const bool ua = J.fock[size_t(w) * 2 * Ns + E.x] >= 0, ub = J.fock[size_t(w) * 2 * Ns + E.y] >= 0;
                anti = ua != ub;
                s0 = ua ? E.x : E.y;
                t0 = ua ? E.y : E.x;
            }
            const unsigned bal = __ballot_sync(0xffffffffu, anti);
            if (lane == 0) s_cnt[warp] = __popc(bal);
            __syncthreads();
            int off = nanti, tot = 0;
            for (int q = 0; q < kTcBlock / 32; ++q) {
                if (q < warp) off += s_cnt[q];
                tot += s_cnt[q];
            }
            if (anti) {
                const int b = off + __popc(bal & ((1u << lane) - 1u));
                s_bs[b] = int16_t(t0);                  // flavour 0 moves s0 -> t0
                s_bs[2 * kOccMaxNs + b] = int16_t(s0);  // flavour 1 moves t0 -> s0
            }
            nanti += tot;
            __syncthreads();
        }
        const cx<float>* cg = J.coef32 + size_t(w) * 4 * Ns;   // [fl][sub][orbital]
        for (int i = tid; i < 2 * N; i += kTcBlock) {
            const int fl = i / N, f = i % N;
            const int o = J.worb[(size_t(w) * 2 + fl) * Nmax + f];
            s_pcol[fl * kTcM + f] = int16_t(o >> 1);
            s_cf[(fl * 2 + 0) * kTcM + f] = cg[(size_t(fl) * 2 + 0) * Ns + o];
            s_cf[(fl * 2 + 1) * kTcM + f] = cg[(size_t(fl) * 2 + 1) * Ns + o];
        }
        __syncthreads();
    };
    // pass p = (fl, bond chunk bc, orbital tile mt), mt fastest
    auto pass_of = [&](int p, int& fl, int& bc, int& mt) {
        const int nbc = (nanti + kTcM - 1) / kTcM;
        mt = p % MT;
        bc = (p / MT) % nbc;
        fl = p / (MT * nbc);
    };
    auto fetch = [&](TcRegs& R, int w, int p, int kc) {
        if (!worker) return;
        int fl, bc, mt;
        pass_of(p, fl, bc, mt);
        const cx<float>* Rf = static_cast<const cx<float>*>(J.gup) + (size_t(w) * 2 + fl) * size_t(Nmax) * Ns;
        tc_load_rows(R, Rf + 2 * mt * kTcM + 1, Ns, min(kTcM, No - mt * kTcM), N, kTcM, kc, 2);
        tc_load_phase_cols(R, J.phase32, Nk, s_bs + fl * 2 * kOccMaxNs + bc * kTcM, s_pcol + fl * kTcM,
                           min(kTcM, nanti - bc * kTcM), N, kTcM, kc);
    };

    TcRegs R;
    int wf = -1;   // the walker whose wait ran out
    for (int w = blockIdx.x; w < J.W && !failed; w += gridDim.x) {
        if (J.status[w] != GV_OK) continue;
        tables(w);
        const int P = 2 * ((nanti + kTcM - 1) / kTcM) * MT;   // passes of this walker
        if (P == 0) continue;
        fetch(R, w, 0, 0);
        bool first = true;
        for (int p = 0; p < P && !failed; ++p) {
            int fl, bc, mt;
            pass_of(p, fl, bc, mt);
            const int nr = min(kTcM, nanti - bc * kTcM);
            for (int kc = 0; kc < KC; ++kc) {
                if (!first) {   // the previous chunk's MMAs are done with the tiles
                    const bool ok = mbar_wait(bar, parity, J.wait_limit);
                    if (__syncthreads_or(!ok)) { failed = true; break; }
                    parity ^= 1u;
                }
                first = false;
                if (worker) {
                    tc_store_inverse(base, lay.a, R, kTcM);
                    tc_store_phi_cols(base, lay.b, R, s_cf + fl * 2 * kTcM, kTcM, s_bs + fl * 2 * kOccMaxNs + bc * kTcM,
                                      nr, N, L, kTcM, kc);
                }
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                tmem_fence_before();
                __syncthreads();
                if (tid == kTcIssuer) {
                    tmem_fence_after();
                    tc_issue_chunk(tbase, 0u, sbase, lay, idesc, kc == 0);
                    tc_commit(bar);
                }
                if (kc + 1 < KC) fetch(R, w, p, kc + 1);
                else if (p + 1 < P) fetch(R, w, p + 1, 0);
            }
            if (failed) break;
            {
                const bool ok = mbar_wait(bar, parity, J.wait_limit);
                if (__syncthreads_or(!ok)) { failed = true; break; }
                parity ^= 1u;
            }
            tmem_fence_after();
            // epilogue: lane o of TMEM -> Z[w][fl][b][o], 16 bonds at a time
            const int lg = warp & 3, oi = mt * kTcM + 32 * lg + lane;
            cx<float>* Zw = Z + (size_t(w) * 2 + fl) * size_t(Bmax) * No;
            for (int cc = warp >> 2; worker && cc < kTcM / 16; cc += 2) {
                if (16 * cc >= nr) break;
                uint32_t r[32];
                const uint32_t ta = tbase + (uint32_t(32 * lg) << 16) + uint32_t(16 * cc);
                tmem_ld16(ta, r);
                tmem_ld16(ta + 128, r + 16);
                tmem_wait_ld(r);
                if (oi < No) {
#pragma unroll
                    for (int t = 0; t < 16; ++t) {
                        const int bl = 16 * cc + t;
                        if (bl < nr)
                            Zw[size_t(bc * kTcM + bl) * No + oi] = cx<float>{__uint_as_float(r[t]), __uint_as_float(r[16 + t])};
                    }
                }
            }
            tmem_fence_before();
            first = true;   // the next pass's first MMAs follow the __syncthreads of its first chunk
        }
        if (failed) {
            wf = w;
            if (tid == 0) J.status[w] = GV_ERR_TIMEOUT;
        }
        __syncthreads();   // the tables of the next walker
    }
    if (failed && tid == 0) tc_mark_rest(J, wf);
    if (failed) mbar_wait(bar, parity);   // the phase that timed out: MMAs in flight finish before TMEM is freed
    tmem_fence_before();
    __syncthreads();
    tmem_fence_after();
    if (warp == 0) tmem_dealloc(tbase, 256);
}

// Occupation bitsets of the walkers still running, word-major: bit b of word
// [fl][k][site] is set when walker 32 k + b holds flavour fl at the site.  One
// block per word k: the 32 walkers' flavour-0 occupancies are staged in
// shared memory by coalesced row loads, then thread i packs site i's bits.
// (Every site of a running walker holds one flavour, so flavour 1's bits are
// the running walkers without flavour 0.)

__global__ void k_occ_bits(DevJob J, uint32_t* bits)
{
    __shared__ int16_t s_f0[32][kOccMaxNs];
    __shared__ int s_run[32];
    const int nw = (J.W + 31) / 32, Ns = J.Ns, k = blockIdx.x;
    if (threadIdx.x < 32) {
        const int w = 32 * k + threadIdx.x;
        s_run[threadIdx.x] = w < J.W && J.status[w] == GV_OK;
    }
    for (int b = 0; b < 32; ++b) {
        const int w = 32 * k + b;
        if (w >= J.W) break;
        for (int i = threadIdx.x; i < Ns; i += blockDim.x) s_f0[b][i] = J.fock[size_t(w) * 2 * Ns + i];
    }
    __syncthreads();
    for (int i = threadIdx.x; i < Ns; i += blockDim.x) {
        uint32_t u = 0, d = 0;
        for (int b = 0; b < 32; ++b) {
            if (!s_run[b]) continue;
            if (s_f0[b][i] >= 0) u |= 1u << b;
            else d |= 1u << b;
        }
        bits[size_t(k) * Ns + i] = u;
        bits[size_t(nw + k) * Ns + i] = d;
    }
}

// Aud[i][j] += number of running walkers with flavour 0 at site i and
// flavour 1 at site j (one thread per entry, so no atomics): the
// antiparallel counts of StatSpinStruct without one atomic per pair.  Block
// i; the flavour-1 words of consecutive sites j are contiguous.
__global__ void k_occ_pairs(DevJob J, const uint32_t* bits)
{
    const int nw = (J.W + 31) / 32, Ns = J.Ns, i = blockIdx.x;
    double* Aud = J.ss + 2 * size_t(Ns) * Ns;
    for (int j = threadIdx.x; j < Ns; j += blockDim.x) {
        int c = 0;
        for (int k = 0; k < nw; ++k) c += __popc(bits[size_t(k) * Ns + i] & bits[size_t(nw + k) * Ns + j]);
        if (c) Aud[size_t(i) * Ns + j] += double(c);
    }
}

}  // namespace
}  // namespace gv
