// Exciton-channel Metropolis walk with its working set on chip (mixed
// precision, Nexc <= 128, N1 <= 127, N0 <= 129: L <= 16).  Included by
// engine.cu after kernels_trans.cuh and kernels_res.cuh.
//
// The streaming exciton kernel (k_walk_trans) re-reads the overlap rows GupT
// (N0 x Nexc, 132 KB at L = 16) and both inverses from L2 / HBM on every
// proposal and accepted move; with two walkers per SM it is latency-bound.
// Here one CTA per SM owns one walker for a whole walk call:
//   TMEM (128 lanes x 512 columns):  GupT^T, lane k = channel state k, Slater
//     row f < 128 in columns 2f, 2f+1, and AiT1, lane f = row f of the
//     flavour-1 inverse, particle p in columns 256 + 2p, 256 + 2p + 1;
//   shared memory: AiT0 (N0 x N0 complex, 133 KB at L = 16), row-major, and
//     GupT's row 128 (N0 = 129), one entry per state.
// The step is k_walk_trans's (same formulas, linalg::DetUpdate / InvUpdate
// restated for the exciton channel), with the per-state overlap
// Z_k = sum_f GupT[f][k] C0[f] a lane-local dot product over a TMEM row, the
// flavour-1 column products summed over lanes by butterfly reduce-scatters,
// and every rank-1 / rank-2 update applied in place on chip.
#pragma once

#include "kernels_res.cuh"
#include "kernels_trans.cuh"

namespace gv {
namespace {

constexpr int kTrThreads = 256;
constexpr size_t kTrMinSmem = 116 * 1024;   // over half an SM's shared memory: one CTA per SM
constexpr uint32_t kA1Col = 256;            // first TMEM column of AiT1
constexpr int kTrBatch = 8;                 // steps per uniform batch (phase rows staged per batch)
constexpr int kTrAccCap = 64;               // accepted ratio pairs held before their product is taken

__host__ __device__ inline bool trans_res_fits(int N0, int N1, int Nexc)
{
    return Nexc <= 128 && N1 <= 127 && N0 <= 129;
}

// Column p of AiT0 in shared memory: sum_f AiT0[f][p] v[f], four independent
// accumulators (short dependency chains), 8 loads in flight.
__device__ __forceinline__ cx<float> smem_col_dot(const cx<float>* A, int N, int p, const cx<float>* v)
{
    cx<float> acc[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
    int f = 0;
    for (; f + 8 <= N; f += 8) {
        cx<float> a[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) a[k] = A[size_t(f + k) * N + p];
#pragma unroll
        for (int k = 0; k < 8; ++k) cmac(acc[k & 3], a[k], v[f + k]);
    }
    for (; f < N; ++f) cmac(acc[0], A[size_t(f) * N + p], v[f]);
    return (acc[0] + acc[1]) + (acc[2] + acc[3]);
}

struct TrResLayout {
    size_t a0, g128, fock, part, wslot, worb, nbr, exu, exd, coef, C, rowc, g, Y, zp, phk, ru, rd, dk, ak, bk, X, Yv, zc,
        hrow, wpart, wa, red, brv, bu4, bu4d, bph, bacc, bbar, tbase, total, used;
};

__host__ __device__ inline TrResLayout trans_res_layout(int Ns, int Nk, int Nmax, int N0, int Nexc)
{
    TrResLayout l;
    size_t b = 0;
    auto al = [&](size_t x) { b = (b + 15) & ~size_t(15); size_t r = b; b += x; return r; };
    const size_t c = sizeof(cx<float>);
    l.a0 = al(c * N0 * N0);
    l.g128 = al(c * 128);
    l.fock = al(sizeof(int16_t) * 2 * Ns);
    l.part = al(sizeof(int16_t) * 2 * Nmax);
    l.wslot = al(sizeof(int16_t) * 2 * Ns);
    l.worb = al(sizeof(int16_t) * 2 * Nmax);
    l.nbr = al(sizeof(int16_t) * 4 * Ns);
    l.exu = al(sizeof(int16_t) * Nexc);
    l.exd = al(sizeof(int16_t) * Nexc);
    l.coef = al(c * 4 * Ns);
    l.C = al(c * 2 * Nmax);
    l.rowc = al(c * 2 * Nmax);
    l.g = al(c * Nmax);
    l.Y = al(c * Nexc);
    l.zp = al(c * Nexc);
    l.phk = al(c * Nexc);
    l.ru = al(c * Nexc);
    l.rd = al(c * Nexc);
    l.dk = al(c * Nexc);
    l.ak = al(c * Nexc);
    l.bk = al(c * Nexc);
    l.X = al(c * 2 * Nmax);
    l.Yv = al(c * 2 * Nmax);
    l.zc = al(c * Nmax);
    l.hrow = al(c * 128);
    l.wpart = al(c * 4 * 128);
    l.wa = al(c * 128);
    l.red = al(sizeof(float) * 2 * 8 * (kTrThreads / 32) + sizeof(int) * (kTrThreads / 32) + 64);
    l.brv = al(sizeof(int16_t) * 3 * 2 * kTrBatch);            // [batch % 3][step][v1, v2]
    l.bu4 = al(sizeof(float) * 3 * kTrBatch);
    l.bu4d = al(sizeof(double) * 3 * kTrBatch);
    l.bph = al(c * 2 * 2 * kTrBatch * size_t(Nk));             // [batch parity][2 step + site][Nk] phase rows
    l.bacc = al(c * 2 * kTrAccCap);                            // accepted ratio pairs not yet in the amplitude
    l.bbar = al(sizeof(uint64_t) * 2);                         // the row buffers' mbarriers
    l.tbase = al(16);
    l.used = al(16);
    l.total = l.used < kTrMinSmem ? kTrMinSmem : l.used;
    return l;
}

__global__ void __launch_bounds__(kTrThreads, 1) k_walk_trans_res(DevJob J, uint64_t nsteps)
{
    extern __shared__ __align__(16) char smem[];
    using T = float;
    constexpr int NT = kTrThreads, NW = NT / 32;
    const int w = blockIdx.x;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (w >= J.W || J.status[w] != GV_OK) return;   // before any TMEM allocation
    const int Ns = J.Ns, Nmax = J.Nmax, L = J.L, Nk = J.Nk, Nexc = J.Nexc;
    const int N0 = J.N[0], N1 = J.N[1];
    const TrResLayout lay = trans_res_layout(Ns, Nk, Nmax, N0, Nexc);
    cx<T>* A0s = reinterpret_cast<cx<T>*>(smem + lay.a0);
    cx<T>* s_g128 = reinterpret_cast<cx<T>*>(smem + lay.g128);   // GupT[128][k]
    int16_t* s_fock = reinterpret_cast<int16_t*>(smem + lay.fock);
    int16_t* s_part = reinterpret_cast<int16_t*>(smem + lay.part);
    int16_t* s_wslot = reinterpret_cast<int16_t*>(smem + lay.wslot);
    int16_t* s_worb = reinterpret_cast<int16_t*>(smem + lay.worb);
    int16_t* s_nbr = reinterpret_cast<int16_t*>(smem + lay.nbr);
    int16_t* s_exu = reinterpret_cast<int16_t*>(smem + lay.exu);
    int16_t* s_exd = reinterpret_cast<int16_t*>(smem + lay.exd);
    cx<T>* s_coef = reinterpret_cast<cx<T>*>(smem + lay.coef);
    cx<T>* s_C = reinterpret_cast<cx<T>*>(smem + lay.C);
    cx<T>* s_rowc = reinterpret_cast<cx<T>*>(smem + lay.rowc);
    cx<T>* s_g = reinterpret_cast<cx<T>*>(smem + lay.g);
    cx<T>* s_Y = reinterpret_cast<cx<T>*>(smem + lay.Y);
    cx<T>* s_zp = reinterpret_cast<cx<T>*>(smem + lay.zp);
    cx<T>* s_phk = reinterpret_cast<cx<T>*>(smem + lay.phk);
    cx<T>* s_ru = reinterpret_cast<cx<T>*>(smem + lay.ru);
    cx<T>* s_rd = reinterpret_cast<cx<T>*>(smem + lay.rd);
    cx<T>* s_dk = reinterpret_cast<cx<T>*>(smem + lay.dk);
    cx<T>* s_ak = reinterpret_cast<cx<T>*>(smem + lay.ak);
    cx<T>* s_bk = reinterpret_cast<cx<T>*>(smem + lay.bk);
    cx<T>* s_X = reinterpret_cast<cx<T>*>(smem + lay.X);
    cx<T>* s_Yv = reinterpret_cast<cx<T>*>(smem + lay.Yv);
    cx<T>* s_zc = reinterpret_cast<cx<T>*>(smem + lay.zc);
    cx<T>* s_hrow = reinterpret_cast<cx<T>*>(smem + lay.hrow);
    cx<T>* s_wpart = reinterpret_cast<cx<T>*>(smem + lay.wpart);
    cx<T>* s_wa = reinterpret_cast<cx<T>*>(smem + lay.wa);
    T* s_red = reinterpret_cast<T*>(smem + lay.red);
    uint32_t* s_tbase = reinterpret_cast<uint32_t*>(smem + lay.tbase);
    int16_t* b_rv = reinterpret_cast<int16_t*>(smem + lay.brv);
    float* b_u4 = reinterpret_cast<float*>(smem + lay.bu4);
    double* b_u4d = reinterpret_cast<double*>(smem + lay.bu4d);
    cx<T>* b_ph = reinterpret_cast<cx<T>*>(smem + lay.bph);
    cx<T>* b_acc = reinterpret_cast<cx<T>*>(smem + lay.bacc);
    uint64_t* b_bar = reinterpret_cast<uint64_t*>(smem + lay.bbar);
    const uint32_t rbar0 = smem_u32(b_bar);

    if (warp == 0) tmem_alloc(s_tbase, 512);
    if (tid == 32) {
        mbar_init(rbar0, 1);
        mbar_init(rbar0 + 8, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    for (int i = tid; i < 2 * Ns; i += NT) {
        s_fock[i] = J.fock[size_t(w) * 2 * Ns + i];
        s_wslot[i] = J.wslot[size_t(w) * 2 * Ns + i];
    }
    for (int i = tid; i < 2 * Nmax; i += NT) {
        s_part[i] = J.part[size_t(w) * 2 * Nmax + i];
        s_worb[i] = J.worb[size_t(w) * 2 * Nmax + i];
    }
    for (int i = tid; i < 4 * Ns; i += NT) s_nbr[i] = int16_t(J.nbr[i]);
    for (int i = tid; i < Nexc; i += NT) { s_exu[i] = J.exc_up[i]; s_exd[i] = J.exc_dn[i]; }
    {
        const cx<T>* cg = J.coef32 + size_t(w) * 4 * Ns;   // [fl][sub][orbital]
        for (int i = tid; i < 4 * Ns; i += NT) s_coef[i] = cg[i];
    }
    cx<T>* A0 = ai_ptr<T>(J, 0, w);
    cx<T>* A1 = ai_ptr<T>(J, 1, w);
    cx<T>* G = static_cast<cx<T>*>(J.gup) + size_t(w) * N0 * Nexc;
    cx<T>* gglob = static_cast<cx<T>*>(J.gdn) + size_t(w) * Nmax;
    for (int i = tid; i < N0 * N0; i += NT) A0s[i] = A0[i];
    for (int i = tid; i < N1; i += NT) s_g[i] = gglob[i];
    if (N0 > 128)
        for (int k = tid; k < Nexc; k += NT) s_g128[k] = G[size_t(128) * Nexc + k];
    for (int i = tid; i < 128; i += NT) s_hrow[i] = cx<T>{T(0), T(0)};   // read (times 0) before a first row change
    tmem_fence_before();
    __syncthreads();
    tmem_fence_after();
    const uint32_t tbase = *s_tbase;
    const int g = tid >> 7;         // warpgroup: 0 serves GupT (lane = state k), 1 serves AiT1 (lane = row f)
    const int lf = tid & 127;       // this thread's TMEM lane
    const int q4 = warp & 3;
    const uint32_t tl = tbase + ((uint32_t(q4) * 32) << 16);
    // overlap rows and the flavour-1 inverse -> TMEM (zero padding)
    if (g == 0) {
        for (int c = 0; c < 4; ++c) {
            uint32_t r[64];
#pragma unroll
            for (int j = 0; j < 32; ++j) {
                const int f = 32 * c + j;
                cx<T> a = {0.f, 0.f};
                if (lf < Nexc && f < N0) a = G[size_t(f) * Nexc + lf];
                r[2 * j] = __float_as_uint(a.x);
                r[2 * j + 1] = __float_as_uint(a.y);
            }
            tmem_st64(tl + 64 * c, r);
        }
    } else {
        for (int c = 0; c < 4; ++c) {
            uint32_t r[64];
#pragma unroll
            for (int j = 0; j < 32; ++j) {
                const int p = 32 * c + j;
                cx<T> a = {0.f, 0.f};
                if (lf < N1 && p < N1) a = A1[size_t(lf) * N1 + p];
                r[2 * j] = __float_as_uint(a.x);
                r[2 * j + 1] = __float_as_uint(a.y);
            }
            tmem_st64(tl + kA1Col + 64 * c, r);
        }
    }
    tmem_wait_st();
    tmem_fence_before();
    __syncthreads();
    tmem_fence_after();

    const cx<T>* phase = J.phase32;
    const cx<T>* cf0 = s_coef;
    const cx<T>* cf1 = s_coef + 2 * Ns;
    const uint32_t wid = J.walker_base + uint32_t(w);
    uint64_t kk = J.rng_next[w];
    unsigned long long c_acc = 0, c_noop = 0, c_rej = 0;
    int since = J.since_reinv[w];
    cx<double> am = J.amp_m[w];
    int ae = J.amp_e[w];
    int cur = J.cur[w];
    int wsign = J.wsign[w];
    double sigma = J.sigma[w];
    int status = GV_OK;
    int rbuf = 0;
    // Uniform batches of kTrBatch steps: warp 0 draws batch b + 2 while the
    // phase rows phi(v1), phi(v2) of batch b + 1 (drawn a batch earlier) come
    // into shared memory as bulk copies on that buffer's mbarrier, so that no
    // step computes Philox numbers or reads the phase table in global memory
    // (every site a step's formulas name is v1 or v2).
    const uint64_t kk0 = kk;
    auto draw_batch = [&](uint64_t sb, int rs) {   // warp 0; a step past the call's end gets sites (0, 0)
        if (lane < kTrBatch) {
            int a1 = 0, a2 = 0;
            float u = 0.f;
            double ud = 0.0;
            if (sb + lane < nsteps) {
                const uint64_t kl = kk0 + 4 * (sb + uint64_t(lane));
                uint32_t x[4], y[4];
                philox_call(J.seed, wid, 0, kl >> 1, x);
                philox_call(J.seed, wid, 0, (kl >> 1) + 1, y);
                a1 = scaled_floor(uint32_t(Ns), u52(x[0], x[1]));
                a2 = s_nbr[a1 * 4 + int(u52(x[2], x[3]) >> 50)];
                u = Accept<T>::uniform(u52(y[2], y[3]));
                if (J.trace) ud = u01(y[2], y[3]);
            }
            b_rv[(rs * kTrBatch + lane) * 2] = int16_t(a1);
            b_rv[(rs * kTrBatch + lane) * 2 + 1] = int16_t(a2);
            b_u4[rs * kTrBatch + lane] = u;
            b_u4d[rs * kTrBatch + lane] = ud;
        }
    };
    auto fetch_rows = [&](int rs, int par) {   // threads 0 .. 2 kTrBatch - 1: one row (8 Nk bytes) each
        const uint32_t bar = rbar0 + 8 * par, rowb = uint32_t(Nk) * 8u;
        if (tid == 0) mbar_expect_tx(bar, uint32_t(2 * kTrBatch) * rowb);
        if (tid < 2 * kTrBatch) {
            const int site = b_rv[(rs * kTrBatch + (tid >> 1)) * 2 + (tid & 1)];
            fence_proxy_async();
            bulk_g2s(smem_u32(b_ph + (size_t(par) * 2 * kTrBatch + tid) * Nk), phase + size_t(site) * Nk, rowb, bar);
        }
    };
    // The amplitude's FP64 products of the accepted ratio pairs, as a warp tree
    // once the pairs' buffer could fill within the next batch and at the end
    // (thread 0 holds the amplitude)
    int nacc = 0;
    auto flush_amp = [&]() {
        if (warp == 0) {
            cx<double> v = {1.0, 0.0};
            int e = 0;
            for (int i = lane; i < nacc; i += 32) {
                v = v * (to_d(b_acc[2 * i]) * to_d(b_acc[2 * i + 1]));
                amp_normalise(v, e);
            }
#pragma unroll
            for (int o = 16; o; o >>= 1) {
                const cx<double> u = {__shfl_xor_sync(0xffffffffu, v.x, o), __shfl_xor_sync(0xffffffffu, v.y, o)};
                e += __shfl_xor_sync(0xffffffffu, e, o);
                v = v * u;
                amp_normalise(v, e);
            }
            if (lane == 0) {
                am = am * v;
                ae += e;
                amp_normalise(am, ae);
            }
        }
        nacc = 0;
    };
    uint32_t nb_issued = 0, nb_waited = 0;
    int rs_cur = 0;
    if (warp == 0) {
        draw_batch(0, 0);
        draw_batch(kTrBatch, 1);
    }
    __syncthreads();
    fetch_rows(0, 0);
    nb_issued = 1;

    for (uint64_t s = 0; s < nsteps; ++s, kk += 4) {
        const int bi = int(s % kTrBatch);
        const int par = int(s / kTrBatch) & 1;
        if (bi == 0) {
            if (s > 0) rs_cur = rs_cur == 2 ? 0 : rs_cur + 1;
            const int rs1 = rs_cur == 2 ? 0 : rs_cur + 1, rs2 = rs1 == 2 ? 0 : rs1 + 1;
            __syncthreads();   // every thread is done with batch b - 1 and its buffers
            if (nacc > kTrAccCap - kTrBatch) flush_amp();
            fetch_rows(rs1, par ^ 1);
            if (warp == 0) draw_batch(s + 2 * kTrBatch, rs2);
            ++nb_issued;
            const bool ok = mbar_wait(rbar0 + 8 * (nb_waited & 1), (nb_waited >> 1) & 1, J.wait_limit);
            ++nb_waited;
            if (__syncthreads_or(!ok)) { status = GV_ERR_TIMEOUT; break; }
        }
        const int v1 = b_rv[(rs_cur * kTrBatch + bi) * 2], v2 = b_rv[(rs_cur * kTrBatch + bi) * 2 + 1];
        const cx<T>* row1 = b_ph + (size_t(par) * 2 * kTrBatch + 2 * bi) * Nk;   // phase row of v1, then of v2
        // phi_o(site) of orbital o from the staged rows (site is v1 or v2)
        auto phi_st = [&](const cx<T>* cfx, int site, int o) {
            const cx<T>* row = site == v1 ? row1 : row1 + Nk;
            return cmul_rn(row[o >> 1], cfx[size_t(sublattice(site, L)) * Ns + o]);
        };
        const int f1 = s_fock[v1] >= 0 ? 0 : 1;
        const int f2 = s_fock[v2] >= 0 ? 0 : 1;
        int kind = 0, accepted, khop = -1;
        T ratio = T(1);
        if (f1 == f2) {
            accepted = 1;
            ++c_noop;
        } else {
            kind = 1;
            const int upf = (f1 == 0) ? v1 : v2, upt = (f1 == 0) ? v2 : v1;
            const int dnf = upt, dnt = upf;
            const int cu = s_fock[upf], cd = s_fock[Ns + dnf];
            const int ocur = s_exu[cur], hcur = s_exd[cur];
            const int r0 = s_wslot[ocur];
            if (r0 < 0) { status = GV_ERR_INVALID; break; }   // Fock state inconsistent with the channel table
            // Phase 1: rows c of both inverses, new columns C, M11 = row_c . C, g . C1,
            // and row r0 of GupT (Y_k).
            cx<T> m11u = {T(0), T(0)}, m11d = {T(0), T(0)}, gc = {T(0), T(0)};
            for (int f = tid; f < N0; f += NT) {
                const cx<T> a = A0s[size_t(f) * N0 + cu];
                const cx<T> c = phi_st(cf0, upt, s_worb[f]);
                s_rowc[f] = a;
                s_C[f] = c;
                cmac(m11u, a, c);
            }
            if (g || r0 < 128) {   // warp-uniform
                uint32_t r2[2];
                tmem_ld2(g ? tl + kA1Col + 2 * cd : tl + 2 * r0, r2);
                tmem_wait_ld(r2);
                const cx<T> v = {__uint_as_float(r2[0]), __uint_as_float(r2[1])};
                if (g) {
                    if (lf < N1) {
                        const cx<T> c = phi_st(cf1, dnt, s_worb[Nmax + lf]);
                        s_rowc[Nmax + lf] = v;
                        s_C[Nmax + lf] = c;
                        cmac(m11d, v, c);
                        cmac(gc, s_g[lf], c);
                    }
                } else if (lf < Nexc) {
                    s_Y[lf] = v;
                }
            } else if (lf < Nexc) {
                s_Y[lf] = s_g128[lf];
            }
            m11u = warp_sum(m11u);
            m11d = warp_sum(m11d);
            gc = warp_sum(gc);
            T* rb = s_red + rbuf * NW * 8;
            rbuf ^= 1;
            if (lane == 0) {
                rb[warp * 8 + 0] = m11u.x; rb[warp * 8 + 1] = m11u.y;
                rb[warp * 8 + 2] = m11d.x; rb[warp * 8 + 3] = m11d.y;
                rb[warp * 8 + 4] = gc.x;   rb[warp * 8 + 5] = gc.y;
            }
            __syncthreads();
            cx<T> M11u = {T(0), T(0)}, M11d = {T(0), T(0)}, gC = {T(0), T(0)};
            for (int q = 0; q < NW; ++q) {
                M11u.x += rb[q * 8 + 0]; M11u.y += rb[q * 8 + 1];
                M11d.x += rb[q * 8 + 2]; M11d.y += rb[q * 8 + 3];
                gC.x += rb[q * 8 + 4];   gC.y += rb[q * 8 + 5];
            }
            // Phase 2: Z_k = sum_f GupT[f][k] C0[f] along lane k's TMEM row; the
            // other warpgroup meanwhile forms phi_{exc_up[k]}(t).
            if (g == 0) {
                cx<T> a4[4] = {{T(0), T(0)}, {T(0), T(0)}, {T(0), T(0)}, {T(0), T(0)}};
                for (int c = 0; c < 4; ++c) {
                    uint32_t r[64];
                    tmem_ld64(tl + 64 * c, r);
                    tmem_wait_ld(r);
                    const cx<T>* cc = s_C + 32 * c;
                    const bool full = 32 * c + 32 <= N0;   // whole chunk inside the matrix (uniform)
#pragma unroll
                    for (int j = 0; j < 32; ++j)
                        if (full || 32 * c + j < N0)
                            cmac(a4[j & 3], cx<T>{__uint_as_float(r[2 * j]), __uint_as_float(r[2 * j + 1])}, cc[j]);
                }
                cx<T> acc = (a4[0] + a4[1]) + (a4[2] + a4[3]);
                if (N0 > 128 && lf < Nexc) cmac(acc, s_g128[lf], s_C[128]);
                if (lf < Nexc) s_zp[lf] = acc;
            } else if (lf < Nexc) {
                s_phk[lf] = phi_st(cf0, upt, s_exu[lf]);
            }
            __syncthreads();
            // Phase 3: per-state ratios, their sum and the first arg-max.
            const cx<T> M12 = s_rowc[r0];
            const cx<T> gcd = gC - phi_st(cf1, dnt, hcur);
            T wsum = T(0), wbest = T(-1);
            int kbest = Nexc;
            for (int k = tid; k < Nexc; k += NT) {
                const cx<T> Z = s_zp[k];
                const cx<T> phk = s_phk[k];
                cx<T> ru = M11u, rd = M11d;
                if (k != cur) {
                    ru = M11u * s_Y[k] - M12 * (Z - phk);
                    const int rk = max(int(s_wslot[Ns + s_exd[k]]), 0);   // occupied for every k != cur
                    rd = M11d * s_g[rk] - s_rowc[Nmax + rk] * gcd;
                }
                s_ru[k] = ru;
                s_rd[k] = rd;
                const T wk = Accept<T>::ratio(ru, rd);
                wsum += wk;
                if (wk > wbest) { wbest = wk; kbest = k; }
            }
#pragma unroll
            for (int o = 16; o; o >>= 1) {
                wsum += __shfl_xor_sync(0xffffffffu, wsum, o);
                const T ob = __shfl_xor_sync(0xffffffffu, wbest, o);
                const int ok = __shfl_xor_sync(0xffffffffu, kbest, o);
                if (ob > wbest || (ob == wbest && ok < kbest)) { wbest = ob; kbest = ok; }
            }
            if (lane == 0) { rb[warp * 8 + 6] = wsum; rb[warp * 8 + 7] = wbest; }
            int* rbi = reinterpret_cast<int*>(s_red + 2 * 8 * NW);   // arg-max indices, after both buffers
            if (lane == 0) rbi[warp] = kbest;
            __syncthreads();
            wsum = T(0);
            wbest = T(-1);
            kbest = Nexc;
            for (int q = 0; q < NW; ++q) {
                wsum += rb[q * 8 + 6];
                if (rb[q * 8 + 7] > wbest || (rb[q * 8 + 7] == wbest && rbi[q] < kbest)) {
                    wbest = rb[q * 8 + 7];
                    kbest = rbi[q];
                }
            }
            khop = kbest;
            ratio = wsum / T(sigma);
            if (!isfinite(ratio) || khop >= Nexc) { status = GV_ERR_NAN; break; }
            accepted = ratio > T(1) ? 1 : (b_u4[rs_cur * kTrBatch + bi] < ratio);
            if (!accepted) {
                ++c_rej;
            } else {
                const cx<T> rho_u = s_ru[khop], rho_d = s_rd[khop];
                if (norm2(rho_u) < T(1e-9) || norm2(rho_d) < T(1e-9)) { status = GV_ERR_SINGULAR; break; }
                const bool row = khop != cur;
                const int rp = row ? max(int(s_wslot[Ns + s_exd[khop]]), 0) : 0;   // flavour-1 row replaced
                // Stage 1: per-state coefficients of the GupT update; GupT's column
                // khop (lane khop's TMEM row) and AiT1's row rp (lane rp's TMEM row)
                // copied to shared memory by their lanes.
                for (int k = tid; k < Nexc; k += NT) {
                    const cx<T> Z = s_zp[k];
                    const cx<T> dk = s_phk[k] - phi_st(cf0, upf, s_exu[k]);
                    s_dk[k] = dk;
                    s_ak[k] = Z + dk * M11u - s_phk[k];
                    s_bk[k] = s_Y[k] + dk * M12;
                }
                if (row) {
                    const int lr = g ? rp : khop;   // the lane whose row is needed
                    if (q4 == (lr >> 5)) {
                        const uint32_t cb = g ? kA1Col : 0u;
                        const int nv = g ? N1 : (N0 < 128 ? N0 : 128);
                        for (int c = 0; c < 4; ++c) {
                            uint32_t r[64];
                            tmem_ld64(tl + cb + 64 * c, r);
                            tmem_wait_ld(r);
                            if (lane == (lr & 31)) {
#pragma unroll
                                for (int j = 0; j < 32; ++j) {
                                    const int i = 32 * c + j;
                                    if (i < nv) {
                                        const cx<T> v = {__uint_as_float(r[2 * j]), __uint_as_float(r[2 * j + 1])};
                                        if (g) s_hrow[i] = v;
                                        else s_zc[i] = v;
                                    }
                                }
                            }
                        }
                        if (g == 0 && N0 > 128 && lane == (lr & 31)) s_zc[128] = s_g128[khop];
                    }
                }
                __syncthreads();
                // Stage 2: capacitance matrices (linalg.cpp:402-573) and the row
                // vectors [X; Y] = M^-1 [row_c; V1] of both flavours.
                cx<T> Mui[4], Mdi[4];
                cx<T> delu = {T(0), T(0)}, deld = {T(0), T(0)}, Dh;
                {
                    const cx<T> phc_t = phi_st(cf1, dnt, hcur);
                    Dh = phc_t - phi_st(cf1, dnf, hcur);
                    if (row) {
                        cx<T> Mu[4], Md[4];
                        delu = s_C[r0] - phi_st(cf0, upf, ocur);
                        const cx<T> Zk = s_zp[khop];
                        const cx<T> dkh = s_dk[khop];
                        const cx<T> raic = Zk + dkh * M11u, raier = s_Y[khop] + dkh * M12;
                        Mu[0] = M11u; Mu[1] = M12;
                        Mu[2] = raic - s_phk[khop] - delu * M11u;
                        Mu[3] = raier - delu * M12;
                        inv2(Mu, Mui);
                        const cx<T> M12d = s_rowc[Nmax + rp];
                        deld = s_C[Nmax + rp] - phi_st(cf1, dnf, s_exd[khop]);
                        const cx<T> raicd = gC + Dh * M11d, raierd = s_g[rp] + Dh * M12d;
                        Md[0] = M11d; Md[1] = M12d;
                        Md[2] = raicd - phc_t - deld * M11d;
                        Md[3] = raierd - deld * M12d;
                        inv2(Md, Mdi);
                    } else {
                        Mui[0] = cinv(M11u);
                        Mdi[0] = cinv(M11d);
                        Mui[1] = Mui[2] = Mui[3] = Mdi[1] = Mdi[2] = Mdi[3] = cx<T>{T(0), T(0)};
                    }
                }
                const cx<T> dkh = row ? s_dk[khop] : cx<T>{T(0), T(0)};
                for (int f = tid; f < N0; f += NT) {
                    const cx<T> rc = s_rowc[f];
                    cx<T> v1 = {T(0), T(0)};
                    if (row) {
                        v1 = s_zc[f] + (dkh - delu) * rc;
                        if (f == r0) v1.x -= T(1);
                    }
                    s_X[f] = Mui[0] * rc + Mui[1] * v1;
                    s_Yv[f] = Mui[2] * rc + Mui[3] * v1;
                }
                for (int f = tid; f < N1; f += NT) {
                    const cx<T> rc = s_rowc[Nmax + f];
                    cx<T> v1 = {T(0), T(0)};
                    if (row) {
                        v1 = s_g[f] + (Dh - deld) * rc;
                        if (f == rp) v1.x -= T(1);
                    }
                    s_X[Nmax + f] = Mdi[0] * rc + Mdi[1] * v1;
                    s_Yv[Nmax + f] = Mdi[2] * rc + Mdi[3] * v1;
                }
                __syncthreads();
                // Stage 3: rank-2 updates.  AiT0 in shared memory, one column per
                // thread: its entry in row r0 before the update, (A^-1 C)_p - [p == c].
                if (g == 0) {
                    const int p = tid;
                    if (p < N0) {
                        const cx<T> h = row ? A0s[size_t(r0) * N0 + p] : cx<T>{T(0), T(0)};
                        cx<T> wa = smem_col_dot(A0s, N0, p, s_C);
                        if (p == cu) wa.x -= T(1);
                        col_update2<T>(A0s, N0, p, wa, s_X, h, s_Yv, row);
                    }
                } else if (N0 > 128 && warp == 5) {
                    // column 128 by one warp of the other warpgroup: rows split over lanes
                    const cx<T> h = row ? A0s[size_t(r0) * N0 + 128] : cx<T>{T(0), T(0)};
                    cx<T> wa = {T(0), T(0)};
                    for (int f = lane; f < N0; f += 32) cmac(wa, A0s[size_t(f) * N0 + 128], s_C[f]);
                    wa = warp_sum(wa);   // every lane has read its rows before any lane writes
                    if (cu == 128) wa.x -= T(1);
                    const cx<T> na = cneg(wa), nb = cneg(h);
                    for (int f = lane; f < N0; f += 32) {
                        cx<T> a = A0s[size_t(f) * N0 + 128];
                        cmac(a, na, s_X[f]);
                        if (row) cmac(a, nb, s_Yv[f]);
                        A0s[size_t(f) * N0 + 128] = a;
                    }
                }
                // GupT[f][k] += d_k row_c[f] - a_k X[f] - b_k Y[f] along lane k's row, 32
                // Slater rows per chunk; either warpgroup can reach every TMEM lane
                // (a warp's lane quarter is warp % 4), so the chunks are shared out
                // to balance the stage: warpgroup 0 also rewrites AiT0, warpgroup 1
                // AiT1
                const bool gok = lf < Nexc;
                const cx<T> gdk = gok ? s_dk[lf] : cx<T>{T(0), T(0)};
                const cx<T> gna = gok ? cneg(s_ak[lf]) : cx<T>{T(0), T(0)};
                const cx<T> gnb = (gok && row) ? cneg(s_bk[lf]) : cx<T>{T(0), T(0)};
                // lanes past Nexc have zero coefficients and are never read
                auto gupt_chunks = [&](int c0, int c1) {
                    for (int c = c0; c < c1; ++c) {
                        uint32_t r[64];
                        tmem_ld64(tl + 64 * c, r);
                        tmem_wait_ld(r);
                        const bool full = 32 * c + 32 <= N0;
#pragma unroll
                        for (int j = 0; j < 32; ++j) {
                            const int f = 32 * c + j;
                            if (full || f < N0) {
                                cx<T> v = {__uint_as_float(r[2 * j]), __uint_as_float(r[2 * j + 1])};
                                cmac(v, gdk, s_rowc[f]);
                                cmac(v, gna, s_X[f]);
                                cmac(v, gnb, s_Yv[f]);   // gnb = 0 without a row change
                                r[2 * j] = __float_as_uint(v.x);
                                r[2 * j + 1] = __float_as_uint(v.y);
                            }
                        }
                        tmem_st64(tl + 64 * c, r);
                    }
                };
                if (g) {
                    // AiT1 in TMEM: (A^-1 C1)_p summed over the lanes f (butterfly per
                    // warp, the four warps in shared memory), then every lane updates
                    // its row: AiT1[f][p] -= wa_p X1[f] + h_p Y1[f].
                    const cx<T> c1 = lf < N1 ? s_C[Nmax + lf] : cx<T>{T(0), T(0)};
                    for (int c = 0; c < 4; ++c) {
                        uint32_t r[64];
                        tmem_ld64(tl + kA1Col + 64 * c, r);
                        tmem_wait_ld(r);
                        cx<T> v[32];
#pragma unroll
                        for (int j = 0; j < 32; ++j) v[j] = cx<T>{__uint_as_float(r[2 * j]), __uint_as_float(r[2 * j + 1])} * c1;
                        s_wpart[q4 * 128 + 32 * c + lane] = warp_reduce_scatter(v);
                    }
                    wg_sync(1);
                    if (lf < N1) {
                        cx<T> wa = s_wpart[lf] + s_wpart[128 + lf] + s_wpart[256 + lf] + s_wpart[384 + lf];
                        if (lf == cd) wa.x -= T(1);
                        s_wa[lf] = wa;
                    }
                    wg_sync(1);
                    const cx<T> nx = lf < N1 ? cneg(s_X[Nmax + lf]) : cx<T>{T(0), T(0)};
                    const cx<T> ny = (row && lf < N1) ? cneg(s_Yv[Nmax + lf]) : cx<T>{T(0), T(0)};
                    for (int c = 0; c < 4; ++c) {
                        uint32_t r[64];
                        tmem_ld64(tl + kA1Col + 64 * c, r);
                        tmem_wait_ld(r);
                        const bool full = 32 * c + 32 <= N1;
#pragma unroll
                        for (int j = 0; j < 32; ++j) {
                            const int p = 32 * c + j;
                            if (full || p < N1) {
                                cx<T> e = {__uint_as_float(r[2 * j]), __uint_as_float(r[2 * j + 1])};
                                cmac(e, s_wa[p], nx);
                                cmac(e, s_hrow[p], ny);   // ny = 0 without a row change
                                r[2 * j] = __float_as_uint(e.x);
                                r[2 * j + 1] = __float_as_uint(e.y);
                            }
                        }
                        tmem_st64(tl + kA1Col + 64 * c, r);
                    }
                    gupt_chunks(2, 4);
                } else {
                    gupt_chunks(0, 2);
                    if (N0 > 128 && gok) {
                        cx<T> v = s_g128[lf];
                        cmac(v, gdk, s_rowc[128]);
                        cmac(v, gna, s_X[128]);
                        if (row) cmac(v, gnb, s_Yv[128]);
                        s_g128[lf] = v;
                    }
                }
                tmem_wait_st();
                __syncthreads();   // the column pass is done with s_C, s_X, s_Yv, s_rowc
                // g of the state after the move (its hole orbital).
                {
                    const cx<T> ah = gC + Dh * M11d - phi_st(cf1, dnt, hcur);
                    const cx<T> M12d = row ? s_rowc[Nmax + rp] : cx<T>{T(0), T(0)};
                    const cx<T> q0 = deld * M11d;
                    cx<T> q1 = deld * M12d;
                    q1.x += T(1);
                    for (int f = tid; f < N1; f += NT) {
                        const cx<T> rc = s_rowc[Nmax + f];
                        cx<T> v;
                        if (row) {
                            v = deld * rc - q0 * s_X[Nmax + f] - q1 * s_Yv[Nmax + f];
                            if (f == rp) v.x += T(1);
                        } else {
                            v = s_g[f] + Dh * rc - ah * s_X[Nmax + f];
                        }
                        s_g[f] = v;
                    }
                }
                // hop sign of the wavefunction (State::HopSign, State.cpp:86-115)
                int hs = 1;
                if (row && warp == 0) {
                    const int n = warp_count_between(s_wslot, ocur, s_exu[khop]) +
                                  warp_count_between(s_wslot + Ns, s_exd[khop], hcur);
                    hs = (n & 1) ? -1 : 1;
                }
                __syncthreads();
                if (tid == 0) {
                    s_fock[upt] = int16_t(cu); s_fock[upf] = -1; s_part[cu] = int16_t(upt);
                    s_fock[Ns + dnt] = int16_t(cd); s_fock[Ns + dnf] = -1; s_part[Nmax + cd] = int16_t(dnt);
                    if (row) {
                        const int onew = s_exu[khop], hnew = s_exd[khop];
                        s_worb[r0] = int16_t(onew); s_wslot[onew] = int16_t(r0); s_wslot[ocur] = -1;
                        s_worb[Nmax + rp] = int16_t(hcur); s_wslot[Ns + hcur] = int16_t(rp); s_wslot[Ns + hnew] = -1;
                    }
                    b_acc[2 * nacc] = rho_u;
                    b_acc[2 * nacc + 1] = rho_d;
                }
                ++nacc;
                if (row) { cur = khop; wsign *= hs; }
                sigma = double(wsum / Accept<T>::ratio(rho_u, rho_d));   // in FP32: only T(sigma) is used
                ++c_acc;
                ++since;
                __syncthreads();
            }
        }
        if (J.trace && w == J.trace_walker && tid == 0) {
            gv_trace t;
            t.v1 = v1; t.v2 = v2; t.kind = kind; t.accepted = accepted; t.khop = kind ? khop : -1; t.pad = 0;
            t.ratio = double(ratio); t.u4 = b_u4d[rs_cur * kTrBatch + bi];
            J.trace[s] = t;
        }
    }
    // the row copies still in flight land before the block exits (bounded)
    bool drained = true;
    for (; nb_waited < nb_issued; ++nb_waited)
        drained = mbar_wait(rbar0 + 8 * (nb_waited & 1), (nb_waited >> 1) & 1) && drained;
    if (__syncthreads_or(!drained)) status = GV_ERR_TIMEOUT;
    flush_amp();
    // write back: AiT0 from shared memory, GupT and AiT1 from TMEM, the rest
    for (int i = tid; i < N0 * N0; i += NT) A0[i] = A0s[i];
    if (g == 0) {
        for (int c = 0; c < 4; ++c) {
            uint32_t r[64];
            tmem_ld64(tl + 64 * c, r);
            tmem_wait_ld(r);
#pragma unroll
            for (int j = 0; j < 32; ++j) {
                const int f = 32 * c + j;
                if (lf < Nexc && f < N0) G[size_t(f) * Nexc + lf] = cx<T>{__uint_as_float(r[2 * j]), __uint_as_float(r[2 * j + 1])};
            }
        }
        if (N0 > 128 && lf < Nexc) G[size_t(128) * Nexc + lf] = s_g128[lf];
    } else {
        for (int c = 0; c < 4; ++c) {
            uint32_t r[64];
            tmem_ld64(tl + kA1Col + 64 * c, r);
            tmem_wait_ld(r);
#pragma unroll
            for (int j = 0; j < 32; ++j) {
                const int p = 32 * c + j;
                if (lf < N1 && p < N1) A1[size_t(lf) * N1 + p] = cx<T>{__uint_as_float(r[2 * j]), __uint_as_float(r[2 * j + 1])};
            }
        }
    }
    for (int i = tid; i < 2 * Ns; i += NT) {
        J.fock[size_t(w) * 2 * Ns + i] = s_fock[i];
        J.wslot[size_t(w) * 2 * Ns + i] = s_wslot[i];
    }
    for (int i = tid; i < 2 * Nmax; i += NT) {
        J.part[size_t(w) * 2 * Nmax + i] = s_part[i];
        J.worb[size_t(w) * 2 * Nmax + i] = s_worb[i];
    }
    for (int i = tid; i < N1; i += NT) gglob[i] = s_g[i];
    if (tid == 0) {
        J.rng_next[w] = kk;
        unsigned long long* c = J.counts + size_t(w) * 5;
        c[0] += c_acc + c_noop + c_rej;
        c[1] += c_acc;
        c[2] += c_noop;
        c[3] += c_rej;
        J.since_reinv[w] = since;
        J.amp_m[w] = am;
        J.amp_e[w] = ae;
        J.cur[w] = cur;
        J.wsign[w] = wsign;
        J.sigma[w] = sigma;
        J.status[w] = status;
    }
    tmem_fence_before();
    __syncthreads();
    tmem_fence_after();
    if (warp == 0) tmem_dealloc(tbase, 512);
}

}  // namespace
}  // namespace gv
