// Engine kernels (ground-state channel).  Included by engine.cu.
//
// Inverse layout: AiT[f][p] = (A^-1)(p, f) -- row f (orbital row of A) is
// contiguous over particles p.  This is the reference's column-major m_mati
// (m_mati[p + f*N]).  With it the two O(N^2) passes of an accepted move are
// thread-per-particle loops over rows f: every load is coalesced across the
// warp, accumulations stay in registers, and particle p's column is owned
// by one thread in both passes, so the matrix-vector product and the rank-1
// update need no barrier between them.
#pragma once

#include "device.cuh"

namespace gv {
namespace {

template <typename T> struct Tab;
template <> struct Tab<double> {
    static __device__ __forceinline__ const cx<double>* phase(const DevJob& J) { return J.phase64; }
    static __device__ __forceinline__ const cx<double>* coef(const DevJob& J) { return J.coef64; }
};
template <> struct Tab<float> {
    static __device__ __forceinline__ const cx<float>* phase(const DevJob& J) { return J.phase32; }
    static __device__ __forceinline__ const cx<float>* coef(const DevJob& J) { return J.coef32; }
};

template <typename T>
__device__ __forceinline__ cx<T>* ai_ptr(const DevJob& J, int fl, int w)
{
    return static_cast<cx<T>*>(J.Ai[fl]) + size_t(w) * J.N[fl] * J.N[fl];
}

__device__ __forceinline__ int sublattice(int s, int L) { return ((s % L) + (s / L)) & 1; }

// Orbital held by Slater row f of flavour fl: the ground state fills the
// lower band in order (orbital 2f); the exciton channel keeps a per-walker
// table, read from `worb` ([fl][Nmax], a shared-memory copy) when given.
__device__ __forceinline__ int row_orbital(const DevJob& J, const int16_t* worb, int w, int fl, int f)
{
    if (worb) return worb[fl * J.Nmax + f];
    if (J.worb) return J.worb[(size_t(w) * 2 + fl) * J.Nmax + f];
    return 2 * f;
}

// phi_o(s) = phase[s][o/2] * coef[sub(s)][o] (coef_fl: [sub][Ns] for one flavour).
template <typename T>
__device__ __forceinline__ cx<T> phi_orb(const cx<T>* phase, const cx<T>* coef_fl, int Nk, int Ns, int L, int s, int o)
{
    return cmul_rn(phase[size_t(s) * Nk + (o >> 1)], coef_fl[size_t(sublattice(s, L)) * Ns + o]);
}

// Exact FP32 -> FP64 widening in integer arithmetic (FP32 subnormals become
// signed zeros), keeping epilogues off GB300's narrow FP64 pipe: products are
// formed in FP32 and only running sums are FP64.
__device__ __forceinline__ double f32_to_f64(float x)
{
    const uint32_t u = __float_as_uint(x), e = (u >> 23) & 0xFFu;
    uint64_t d = uint64_t(u & 0x80000000u) << 32;
    if (e) d |= (uint64_t(e == 0xFFu ? 0x7FFu : e + 896u) << 52) | (uint64_t(u & 0x7FFFFFu) << 29);
    return __longlong_as_double(static_cast<long long>(d));
}

template <typename T>
__device__ __forceinline__ cx<T> warp_sum(cx<T> v)
{
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
    }
    return v;
}

// phi_{2f}(s) for ground-state row f: phase[s][f] * coef[sub(s)][2f]
// (coef_fl here is the per-row copy [sub][f]).
template <typename T>
__device__ __forceinline__ cx<T> phi_row(const cx<T>* phase, const cx<T>* coef_fl, int Nk, int Nmax, int L, int s,
                                         int f)
{
    return cmul_rn(phase[size_t(s) * Nk + f], coef_fl[sublattice(s, L) * Nmax + f]);
}

// ------------------------------------------------------------------------
// FP64 Gauss-Jordan inversion with partial (row) pivoting on max |re|+|im|,
// in place on M (N x N row-major).  det = prod(pivots) * (-1)^swaps.
struct GJSmem {
    cx<double>* rowk;
    cx<double>* fcol;
    int* perm;
    double* redv;
    int* redi;
    cx<double>* detm;
    int* dete;
    int* flag;
};

template <int NT>
__device__ __forceinline__ GJSmem carve_gj(char*& p, int Nmax)
{
    GJSmem S;
    S.rowk = reinterpret_cast<cx<double>*>(p); p += sizeof(cx<double>) * Nmax;
    S.fcol = reinterpret_cast<cx<double>*>(p); p += sizeof(cx<double>) * Nmax;
    S.detm = reinterpret_cast<cx<double>*>(p); p += sizeof(cx<double>) * 2;
    S.redv = reinterpret_cast<double*>(p); p += sizeof(double) * (NT / 32);
    S.perm = reinterpret_cast<int*>(p); p += sizeof(int) * Nmax;
    S.redi = reinterpret_cast<int*>(p); p += sizeof(int) * (NT / 32);
    S.dete = reinterpret_cast<int*>(p); p += sizeof(int) * 2;
    S.flag = reinterpret_cast<int*>(p); p += sizeof(int) * 2;
    p = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(p) + 15) & ~uintptr_t(15));
    return S;
}

__host__ __device__ inline size_t gj_smem_bytes(int Nmax, int NT)
{
    return sizeof(cx<double>) * (2 * Nmax + 2) + sizeof(double) * (NT / 32) + sizeof(int) * (Nmax + NT / 32 + 4) + 16;
}

template <int NT>
__device__ bool gj_invert(cx<double>* M, int N, const GJSmem& S, cx<double>& det_m, int& det_e)
{
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    constexpr int NW = NT / 32;
    cx<double> dm = {1.0, 0.0};
    int de = 0;
    for (int k = 0; k < N; ++k) {
        double best = -1.0;
        int bi = N;
        for (int i = k + tid; i < N; i += NT) {
            const cx<double> v = M[size_t(i) * N + k];
            const double a = fabs(v.x) + fabs(v.y);
            if (a > best) { best = a; bi = i; }
        }
#pragma unroll
        for (int o = 16; o; o >>= 1) {
            const double ob = __shfl_xor_sync(0xffffffffu, best, o);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
        }
        if (lane == 0) { S.redv[warp] = best; S.redi[warp] = bi; }
        __syncthreads();
        best = S.redv[0];
        bi = S.redi[0];
        for (int q = 1; q < NW; ++q)
            if (S.redv[q] > best || (S.redv[q] == best && S.redi[q] < bi)) { best = S.redv[q]; bi = S.redi[q]; }
        if (!(best > 0.0)) return false;
        const int p = bi;
        if (p != k)
            for (int j = tid; j < N; j += NT) {
                const cx<double> a = M[size_t(k) * N + j];
                M[size_t(k) * N + j] = M[size_t(p) * N + j];
                M[size_t(p) * N + j] = a;
            }
        __syncthreads();
        const cx<double> piv = M[size_t(k) * N + k];
        if (tid == 0) {
            S.perm[k] = p;
            dm = dm * piv;
            if (p != k) { dm.x = -dm.x; dm.y = -dm.y; }
            amp_normalise(dm, de);
        }
        const cx<double> inv = cinv(piv);
        for (int j = tid; j < N; j += NT) {
            cx<double> v = (j == k) ? cx<double>{1.0, 0.0} : M[size_t(k) * N + j];
            S.rowk[j] = v * inv;
        }
        for (int i = tid; i < N; i += NT) S.fcol[i] = (i == k) ? cx<double>{0.0, 0.0} : M[size_t(i) * N + k];
        __syncthreads();
        for (int j = tid; j < N; j += NT) M[size_t(k) * N + j] = S.rowk[j];
        for (int i = warp; i < N; i += NW) {
            if (i == k) continue;
            const cx<double> f = S.fcol[i];
            const cx<double> nf = {-f.x, -f.y};
            for (int j = lane; j < N; j += 32) {
                cx<double> v = (j == k) ? cx<double>{0.0, 0.0} : M[size_t(i) * N + j];
                cmac(v, nf, S.rowk[j]);
                M[size_t(i) * N + j] = v;
            }
        }
        __syncthreads();
    }
    for (int k = N - 1; k >= 0; --k) {
        const int p = S.perm[k];
        if (p != k)
            for (int i = tid; i < N; i += NT) {
                const cx<double> a = M[size_t(i) * N + k];
                M[size_t(i) * N + k] = M[size_t(i) * N + p];
                M[size_t(i) * N + p] = a;
            }
        __syncthreads();
    }
    if (tid == 0) { det_m = dm; det_e = de; }
    return true;
}

// SlaterDeterminant::Init for walker w (SlaterDeterminant.cpp:60-92).
// Inverts M = A^T, M[r][f] = phi_{2f}(site of particle r): M^-1 = (A^-1)^T,
// i.e. M^-1[f][p] = (A^-1)(p, f), already in the AiT layout.  Amplitude =
// det_0 * det_1; singular as linalg::DetInv (|det|^2 < 1e-9) or zero overlap
// (base-10 exponent < -8, SlaterDeterminant.cpp:78-81).
template <typename T, int NT>
__device__ __noinline__ int reinvert_walker(const DevJob& J, int w, cx<double>* M, const GJSmem& S,
                                            const int16_t* part_s, const int16_t* worb_s = nullptr)
{
    const int tid = threadIdx.x;
    cx<double> am = {1.0, 0.0};
    int ae = 0;
    int status = GV_OK;
    for (int fl = 0; fl < 2; ++fl) {
        const int N = J.N[fl];
        const int16_t* part = part_s ? part_s + fl * J.Nmax : J.part + (size_t(w) * 2 + fl) * J.Nmax;
        const cx<double>* coef = J.coef64 + (size_t(w) * 2 + fl) * 2 * J.Ns;
        for (int idx = tid; idx < N * N; idx += NT) {
            const int r = idx / N, f = idx % N;
            const int s = part[r], o = row_orbital(J, worb_s, w, fl, f);
            M[idx] = cmul_rn(J.phase64[size_t(s) * J.Nk + (o >> 1)], coef[size_t(sublattice(s, J.L)) * J.Ns + o]);
        }
        __syncthreads();
        cx<double> dm;
        int de;
        bool ok = gj_invert<NT>(M, N, S, dm, de);
        if (tid == 0) { S.detm[0] = dm; S.dete[0] = de; S.flag[0] = ok; }
        __syncthreads();
        ok = S.flag[0];
        dm = S.detm[0];
        de = S.dete[0];
        __syncthreads();
        const double l10 = ok ? (log10(sqrt(norm2(dm))) + de * 0.30102999566398119521) : -1e300;
        if (!ok || 2.0 * l10 < -9.0 || floor(l10) < -8.0) status = GV_ERR_SINGULAR;
        cx<T>* out = ai_ptr<T>(J, fl, w);
        for (int idx = tid; idx < N * N; idx += NT) {
            const cx<double> v = M[idx];
            out[idx] = cx<T>{T(v.x), T(v.y)};
        }
        am = am * dm;
        ae += de;
        amp_normalise(am, ae);
        __syncthreads();
    }
    if (tid == 0) {
        if (status == GV_OK) { J.amp_m[w] = am; J.amp_e[w] = ae; }
        else { J.amp_m[w] = cx<double>{0.0, 0.0}; J.amp_e[w] = 0; }
    }
    __syncthreads();
    return status;
}

// Exciton channel: rebuild the overlap rows of a freshly inverted walker,
//   GupT[f][k] = sum_p phi_{exc_up[k]}(x_p) (A0^-1)(p, f)   (every candidate upper orbital)
//   g[f]       = sum_p phi_{exc_dn[cur]}(x_p) (A1^-1)(p, f) (the hole orbital of `cur`)
// from the stored inverses, in the walk precision.  These are the
// R A^-1 products of linalg::DetUpdate / InvUpdate (linalg.cpp:107-573) for
// every row a channel-state hop can bring in: with them a proposal costs one
// Nexc x N0 product instead of the reference's full A^-1 C and R (A^-1 C)
// per step.  The FP64 re-inversion scratch holds Phi[p][k] meanwhile.
template <typename T, int NT>
__device__ __noinline__ void trans_rebuild(const DevJob& J, int w, const int16_t* part_s, int cur)
{
    constexpr int NW = NT / 32;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int N0 = J.N[0], N1 = J.N[1], Nexc = J.Nexc, Ns = J.Ns, Nk = J.Nk, L = J.L;
    const int16_t* part0 = part_s ? part_s : J.part + size_t(w) * 2 * J.Nmax;
    const int16_t* part1 = part0 + J.Nmax;
    const cx<T>* phase = Tab<T>::phase(J);
    const cx<T>* cf0 = Tab<T>::coef(J) + size_t(w) * 4 * Ns;
    const cx<T>* cf1 = cf0 + 2 * Ns;
    cx<T>* Phi = reinterpret_cast<cx<T>*>(J.scratch64 + size_t(w) * J.Nmax * J.Nmax);
    for (int idx = tid; idx < N0 * Nexc; idx += NT) {
        const int p = idx / Nexc, k = idx % Nexc;
        Phi[idx] = phi_orb<T>(phase, cf0, Nk, Ns, L, part0[p], J.exc_up[k]);
    }
    __syncthreads();
    const cx<T>* A0 = ai_ptr<T>(J, 0, w);
    cx<T>* G = static_cast<cx<T>*>(J.gup) + size_t(w) * N0 * Nexc;
    for (int idx = tid; idx < N0 * Nexc; idx += NT) {
        const int f = idx / Nexc, k = idx % Nexc;
        cx<T> acc = {T(0), T(0)};
        for (int p = 0; p < N0; ++p) cmac(acc, Phi[size_t(p) * Nexc + k], A0[size_t(f) * N0 + p]);
        G[idx] = acc;
    }
    const int hole = J.exc_dn[cur];
    const cx<T>* A1 = ai_ptr<T>(J, 1, w);
    cx<T>* g = static_cast<cx<T>*>(J.gdn) + size_t(w) * J.Nmax;
    for (int f = warp; f < N1; f += NW) {
        cx<T> acc = {T(0), T(0)};
        for (int p = lane; p < N1; p += 32)
            cmac(acc, phi_orb<T>(phase, cf1, Nk, Ns, L, part1[p], hole), A1[size_t(f) * N1 + p]);
        acc = warp_sum(acc);
        if (lane == 0) g[f] = acc;
    }
    __syncthreads();
}

// Longitudinal exciton channel: rebuild R of both flavours of a freshly inverted walker from its stored
// inverses: R[f][o] = sum_p phi_o(x_p) (A^-1)(p, f) for every orbital o
// (the R A^-1 products of linalg::DetUpdate for every row a state can bring in).
template <typename T, int NT>
__device__ __noinline__ void long_rebuild(const DevJob& J, int w, const int16_t* part_s)
{
    const int N = J.N[0], Ns = J.Ns, Nk = J.Nk, L = J.L;
    const cx<T>* phase = Tab<T>::phase(J);
    for (int fl = 0; fl < 2; ++fl) {
        const int16_t* part = part_s ? part_s + fl * J.Nmax : J.part + (size_t(w) * 2 + fl) * J.Nmax;
        const cx<T>* cf = Tab<T>::coef(J) + (size_t(w) * 2 + fl) * 2 * Ns;
        const cx<T>* A = ai_ptr<T>(J, fl, w);
        cx<T>* R = static_cast<cx<T>*>(J.gup) + (size_t(w) * 2 + fl) * size_t(J.Nmax) * Ns;
        for (int idx = threadIdx.x; idx < N * Ns; idx += NT) {
            const int f = idx / Ns, o = idx % Ns;
            cx<T> acc = {T(0), T(0)};
            for (int p = 0; p < N; ++p) cmac(acc, phi_orb<T>(phase, cf, Nk, Ns, L, part[p], o), A[size_t(f) * N + p]);
            R[idx] = acc;
        }
    }
    __syncthreads();
}

// Initial inversion / re-inversion of every walker (only_due: only walkers
// whose accepted-move count reached reinv_every, the deferred cadence).
// m_in_smem: the Gauss-Jordan working matrix in shared memory (the launch
// provides Nmax^2 complex FP64 after the GJ scratch) instead of the global
// scratch, for matrices that fit: the N pivot passes then never leave the SM.
template <typename T, int NT>
__global__ void __launch_bounds__(NT) k_invert(DevJob J, int only_due, int m_in_smem)
{
    extern __shared__ __align__(16) char smem[];
    const int w = blockIdx.x;
    if (w >= J.W) return;
    if (only_due) {
        if (J.status[w] != GV_OK || J.reinv_every <= 0 || J.since_reinv[w] < J.reinv_every) return;
    }
    char* p = smem;
    GJSmem S = carve_gj<NT>(p, J.Nmax);
    cx<double>* M = m_in_smem ? reinterpret_cast<cx<double>*>(p) : J.scratch64 + size_t(w) * J.Nmax * J.Nmax;
    const int st = reinvert_walker<T, NT>(J, w, M, S, nullptr);
    if (J.channel == GV_CH_TRANS && st == GV_OK) trans_rebuild<T, NT>(J, w, nullptr, J.cur[w]);
    if (J.channel == GV_CH_LONG && st == GV_OK) long_rebuild<T, NT>(J, w, nullptr);
    if (threadIdx.x == 0) {
        J.status[w] = st;
        if (only_due) { J.since_reinv[w] = 0; J.counts[size_t(w) * 5 + 4] += 1; }
    }
}

// ------------------------------------------------------------------------
// Metropolis walk, ground-state channel: one CTA per walker.  Each step is
// MetroMC::Step (MetroMC.cpp:90-103): uniforms u1..u4 (vertex, neighbour,
// internal state, accept test); equal flavours are a no-op that is always
// accepted; otherwise the determinant ratios
//     r_fl = sum_f (A^-1)(c, f) phi_{2f}(d)          (linalg.cpp:297-303 / 146)
// and on acceptance the Sherman-Morrison update of both inverses
//     A^-1 <- A^-1 - (A^-1 u - e_c)(e_c^T A^-1) / r  (linalg.cpp:402-573, rc=1).
// The Metropolis ratio |r_0 r_1|^2 and the accept uniform: the plain form in
// FP64 exactly as MetroMC::YesNo compares; the mixed form in FP32 (a 24-bit
// uniform), which keeps the per-step scalar work off the FP64 pipe.
template <typename T> struct Accept;
template <> struct Accept<double> {
    static __device__ __forceinline__ double ratio(cx<double> a, cx<double> b) { return norm2(a * b); }
    static __device__ __forceinline__ double uniform(uint64_t m) { return (double(m) + 0.5) * (1.0 / 4503599627370496.0); }
};
template <> struct Accept<float> {
    static __device__ __forceinline__ float ratio(cx<float> a, cx<float> b) { return norm2(a) * norm2(b); }
    static __device__ __forceinline__ float uniform(uint64_t m)
    {
        return (float(uint32_t(m >> 28)) + 0.5f) * (1.0f / 16777216.0f);
    }
};

struct WalkLayout {
    size_t fock, part, nbr, coef, uu, row, rr, red, rdn, gj, pend, redk, total;
};

template <typename T, int NT, int KD>
__host__ __device__ inline WalkLayout walk_layout(int Ns, int Nmax, bool projheis, bool gj)
{
    WalkLayout l;
    size_t b = 0;
    auto al = [&](size_t x) { b = (b + 15) & ~size_t(15); size_t r = b; b += x; return r; };
    l.fock = al(sizeof(int16_t) * 2 * Ns);
    l.part = al(sizeof(int16_t) * 2 * Nmax);
    l.nbr = al(sizeof(int16_t) * 4 * Ns);
    l.coef = al(sizeof(cx<T>) * 4 * Nmax);
    l.uu = al(sizeof(cx<T>) * 2 * Nmax);
    l.row = al(sizeof(cx<T>) * 2 * Nmax);
    l.rr = al(sizeof(cx<T>) * 2 * Nmax);
    l.red = al(sizeof(double) * (2 * (NT / 32) * 4 + (NT / 32) * 4));
    l.rdn = al(projheis ? sizeof(cx<T>) * 4 * Ns : 16);
    l.gj = al(gj ? gj_smem_bytes(Nmax, NT) : 16);
    // delayed updates: per flavour KD row vectors rr_j[f], KD column vectors w_j[p]
    l.pend = al(KD ? sizeof(cx<T>) * 2 * 2 * KD * Nmax : 16);
    l.redk = al(KD ? sizeof(T) * 4 * KD * (NT / 32) + sizeof(cx<T>) * 2 * KD : 16);
    l.total = al(16);
    return l;
}

// Column p of AiT (rows f = 0..N-1): acc = sum_f AiT[f][p] * v[f], 8 loads in flight.
template <typename T>
__device__ __forceinline__ cx<T> col_dot(const cx<T>* __restrict__ A, int N, int p, const cx<T>* v)
{
    cx<T> acc = {T(0), T(0)};
    int f = 0;
    for (; f + 8 <= N; f += 8) {
        cx<T> a[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) a[k] = A[size_t(f + k) * N + p];
#pragma unroll
        for (int k = 0; k < 8; ++k) cmac(acc, a[k], v[f + k]);
    }
    for (; f < N; ++f) cmac(acc, A[size_t(f) * N + p], v[f]);
    return acc;
}

// Column p of AiT: AiT[f][p] -= w * rr[f], 8 loads in flight.
template <typename T>
__device__ __forceinline__ void col_update(cx<T>* A, int N, int p, cx<T> w, const cx<T>* rr)
{
    const cx<T> nw = {-w.x, -w.y};
    int f = 0;
    for (; f + 8 <= N; f += 8) {
        cx<T> a[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) a[k] = A[size_t(f + k) * N + p];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            cmac(a[k], nw, rr[f + k]);
            A[size_t(f + k) * N + p] = a[k];
        }
    }
    for (; f < N; ++f) {
        cx<T> a = A[size_t(f) * N + p];
        cmac(a, nw, rr[f]);
        A[size_t(f) * N + p] = a;
    }
}

// Pointers a walk CTA keeps for its walker (shared-memory copies and its
// inverses), passed to the measurement code.
template <typename T>
struct WalkCtx {
    const DevJob* J;
    int w, Ns, Nmax, L, Nk, N0, N1;
    int16_t* s_fock;
    int16_t* s_part;
    int16_t* s_nbr;
    cx<T>* s_coef;
    cx<T>* s_rq;
    double* s_redm;
    const cx<T>* phase;
    cx<T>* A0;
    cx<T>* A1;
};

// ProjHeis pass 2 (ProjHeis.cpp:40-158): with every particle's ratio to each
// antiparallel neighbour in rq[site][slot] (a site holds one particle), walk
// the edges in creation order, pair the two flavours' ratios of each
// antiparallel bond and add E/site to the walker's accumulator
// (Quantity::measure, Quantity.cpp:24-27).
template <typename T, int NT>
__device__ void projheis_from_rq(const WalkCtx<T>& C)
{
    constexpr int NW = NT / 32;
    const DevJob& J = *C.J;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int16_t* s_fock = C.s_fock;
    const cx<T>* s_rq = C.s_rq;
    double* s_redm = C.s_redm;
    cx<double> e = {0.0, 0.0};
    for (int ed = tid; ed < 2 * C.Ns; ed += NT) {
        const int4 E = J.edges[ed];   // (i, j, slot of j at i, slot of i at j)
        const bool ui = s_fock[E.x] >= 0, uj = s_fock[E.y] >= 0;
        if (ui == uj) { e.x += 0.25; continue; }
        const cx<double> r = to_d(s_rq[E.x * 4 + E.z]) * to_d(s_rq[E.y * 4 + E.w]);
        e.x += -0.25 - 0.5 * r.x;
        e.y += -0.5 * r.y;
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        e.x += __shfl_xor_sync(0xffffffffu, e.x, o);
        e.y += __shfl_xor_sync(0xffffffffu, e.y, o);
    }
    if (lane == 0) { s_redm[warp * 4] = e.x; s_redm[warp * 4 + 1] = e.y; }
    __syncthreads();
    if (tid == 0) {
        const double inv_ns = 1.0 / double(C.Ns);
        double ex = 0, ey = 0;
        for (int q = 0; q < NW; ++q) { ex += s_redm[q * 4]; ey += s_redm[q * 4 + 1]; }
        J.pj[size_t(C.w) * 2].x += ex * inv_ns;
        J.pj[size_t(C.w) * 2].y += ey * inv_ns;
        J.pj[size_t(C.w) * 2 + 1].x += 1.0;
        J.pj_n[C.w] += 1;
    }
    __syncthreads();
}

// StagMagnZ (StagMagnZ.cpp:12-43) of the walker's current configuration.
template <typename T, int NT>
__device__ void stagmagn_now(const WalkCtx<T>& C)
{
    constexpr int NW = NT / 32;
    const DevJob& J = *C.J;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int L = C.L;
    int m = 0;
    for (int v = tid; v < C.Ns; v += NT) {
        const int sg = (((v % L) + (v / L)) & 1) ? -1 : 1;
        m += sg * (C.s_fock[v] >= 0 ? 1 : -1);
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) m += __shfl_xor_sync(0xffffffffu, m, o);
    if (lane == 0) C.s_redm[warp * 4 + 2] = double(m);
    __syncthreads();
    if (tid == 0) {
        double t = 0;
        for (int q = 0; q < NW; ++q) t += C.s_redm[q * 4 + 2];
        const double inv_ns = 1.0 / double(C.Ns);
        J.sm[C.w].x += t * inv_ns;
        J.sm_n[C.w] += 1;
    }
    __syncthreads();
}

// ProjHeis and StagMagnZ of the walker's current configuration, added to
// its accumulators (Quantity::measure, Quantity.cpp:24-27).  RND rows of the
// inverse per round in pass 1 (more loads in flight for callers with spare
// registers).
template <typename T, int NT, int RND = 1>
__device__ void measure_now(const WalkCtx<T>& C, int mask)
{
    const int tid = threadIdx.x;
    const int Nmax = C.Nmax, L = C.L, Nk = C.Nk, N0 = C.N0, N1 = C.N1;
    const int16_t* s_fock = C.s_fock;
    const int16_t* s_part = C.s_part;
    const int16_t* s_nbr = C.s_nbr;
    const cx<T>* s_coef = C.s_coef;
    cx<T>* s_rq = C.s_rq;
    const cx<T>* phase = C.phase;
    const cx<T>* A0 = C.A0;
    const cx<T>* A1 = C.A1;
    if (mask & GV_MEAS_PROJHEIS) {
        // pass 1: every particle's ratio of moving to each antiparallel neighbour
        for (int idx = tid; idx < N0 + N1; idx += NT) {
            const int fl = idx < N0 ? 0 : 1;
            const int p = fl ? idx - N0 : idx;
            const int N = fl ? N1 : N0;
            const cx<T>* A = fl ? A1 : A0;
            const cx<T>* cf = s_coef + fl * 2 * Nmax;
            const int site = s_part[fl * Nmax + p];
            int js[4];
            bool anti[4];
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
                js[kk] = s_nbr[site * 4 + kk];
                anti[kk] = (s_fock[js[kk]] >= 0) != (fl == 0);
            }
            // phi_{2f}(j) = phase[j][f] coef[sub(j)][f]: per neighbour one phase row and
            // one coefficient row; RND rows f per round keep the loads in flight
            const cx<T>* ph[4];
            const cx<T>* cr[4];
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
                ph[kk] = phase + size_t(js[kk]) * Nk;
                cr[kk] = cf + sublattice(js[kk], L) * Nmax;
            }
            cx<T> acc[4] = {{T(0), T(0)}, {T(0), T(0)}, {T(0), T(0)}, {T(0), T(0)}};
            int f = 0;
            for (; f + RND <= N; f += RND) {
                cx<T> a[RND], q[4][RND];
#pragma unroll
                for (int i = 0; i < RND; ++i) a[i] = A[size_t(f + i) * N + p];
#pragma unroll
                for (int kk = 0; kk < 4; ++kk)
#pragma unroll
                    for (int i = 0; i < RND; ++i) q[kk][i] = anti[kk] ? ph[kk][f + i] : cx<T>{T(0), T(0)};
#pragma unroll
                for (int kk = 0; kk < 4; ++kk)
#pragma unroll
                    for (int i = 0; i < RND; ++i)
                        if (anti[kk]) cmac(acc[kk], a[i], cmul_rn(q[kk][i], cr[kk][f + i]));
            }
            for (; f < N; ++f) {
                const cx<T> a = A[size_t(f) * N + p];
#pragma unroll
                for (int kk = 0; kk < 4; ++kk)
                    if (anti[kk]) cmac(acc[kk], a, cmul_rn(ph[kk][f], cr[kk][f]));
            }
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) s_rq[site * 4 + kk] = acc[kk];
        }
        __syncthreads();
        projheis_from_rq<T, NT>(C);
    }
    if (mask & GV_MEAS_STAGMAGN) stagmagn_now<T, NT>(C);
}

// Pending rank-1 updates (delayed Sherman-Morrison, McDaniel et al., J. Chem.
// Phys. 147, 174107 (2017)): the stored AiT0 lags the current inverse by the
// pending pairs, AiT_cur[f][p] = AiT0[f][p] - sum_j rr_j[f] w_j[p].
template <typename T, int KD>
struct Pending {
    cx<T>* rr;   // [fl][KD][Nmax]
    cx<T>* w;    // [fl][KD][Nmax]
    int n;
};

// Write the pending pairs into AiT0 (one read + write pass per column).
template <typename T, int NT, int KD>
__device__ __forceinline__ void flush_pending(Pending<T, KD>& P, cx<T>* A0, cx<T>* A1, int N0, int N1, int Nmax)
{
    if constexpr (KD == 0) {
        return;
    } else {
        if (P.n == 0) return;
        for (int fl = 0; fl < 2; ++fl) {
            const int N = fl ? N1 : N0;
            cx<T>* A = fl ? A1 : A0;
            const cx<T>* rr = P.rr + size_t(fl) * KD * Nmax;
            const cx<T>* wv = P.w + size_t(fl) * KD * Nmax;
            for (int p = threadIdx.x; p < N; p += NT) {
                cx<T> w[KD > 0 ? KD : 1];
#pragma unroll
                for (int j = 0; j < KD; ++j) w[j] = j < P.n ? cx<T>{-wv[j * Nmax + p].x, -wv[j * Nmax + p].y} : cx<T>{T(0), T(0)};
                int f = 0;
                for (; f + 8 <= N; f += 8) {
                    cx<T> a[8];
#pragma unroll
                    for (int q = 0; q < 8; ++q) a[q] = A[size_t(f + q) * N + p];
#pragma unroll
                    for (int q = 0; q < 8; ++q) {
#pragma unroll
                        for (int j = 0; j < KD; ++j)
                            if (j < P.n) cmac(a[q], w[j], rr[j * Nmax + f + q]);   // rows past n are not written yet
                        A[size_t(f + q) * N + p] = a[q];
                    }
                }
                for (; f < N; ++f) {
                    cx<T> a = A[size_t(f) * N + p];
#pragma unroll
                    for (int j = 0; j < KD; ++j)
                        if (j < P.n) cmac(a, w[j], rr[j * Nmax + f]);
                    A[size_t(f) * N + p] = a;
                }
            }
        }
        P.n = 0;
        __syncthreads();
    }
}


// Accepted exchange with delayed updates.  With r the ratio, row_c the
// current row c of A^-1 and u the new orbital column:
//   rr_new = row_c / r,  w_new = A_cur^-1 u - e_c,
//   A_cur^-1 u = AiT0^T u - sum_j w_j (rr_j . u).
// The column pass reads AiT0 once to form AiT0^T u; when the list is full the
// same pass also writes the KD pending pairs into AiT0 (and the new pair
// starts the next list), so the matrix is written once per KD accepts.
template <typename T, int NT, int KD>
__device__ __noinline__ void accept_delayed(Pending<T, KD>& P, cx<T>* A0, cx<T>* A1, int N0, int N1, int Nmax,
                                            int cu, int cd, cx<T> iu, cx<T> id, const cx<T>* s_row,
                                            const cx<T>* s_uu, T* red)
{
    constexpr int NW = NT / 32;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int np = P.n;
    // s_j = rr_j . u for both flavours (block reduction of 2*np complex numbers)
#pragma unroll
    for (int fl = 0; fl < 2; ++fl) {
        const int N = fl ? N1 : N0;
#pragma unroll
        for (int j = 0; j < KD; ++j) {
            cx<T> a = {T(0), T(0)};
            if (j < np)
                for (int f = tid; f < N; f += NT) cmac(a, P.rr[(fl * KD + j) * Nmax + f], s_uu[fl * Nmax + f]);
            a = warp_sum(a);
            if (lane == 0) { red[((fl * KD + j) * NW + warp) * 2] = a.x; red[((fl * KD + j) * NW + warp) * 2 + 1] = a.y; }
        }
    }
    __syncthreads();
    cx<T>* sj = reinterpret_cast<cx<T>*>(red + 4 * KD * NW);   // [fl][KD], after the partials
    if (tid < 2 * KD) {
        cx<T> a = {T(0), T(0)};
        for (int q = 0; q < NW; ++q) { a.x += red[(tid * NW + q) * 2]; a.y += red[(tid * NW + q) * 2 + 1]; }
        sj[tid] = a;
    }
    __syncthreads();
    const bool full = np == KD;
    const int slot = full ? 0 : np;
    // rows rr_new go to the list after the column pass (the pass may still read old rows)
    cx<T> wnew[2];
    int pidx[2];
#pragma unroll
    for (int fl = 0; fl < 2; ++fl) {
        const int N = fl ? N1 : N0;
        cx<T>* A = fl ? A1 : A0;
        const int c = fl ? cd : cu;
        const cx<T>* rr = P.rr + size_t(fl) * KD * Nmax;
        const cx<T>* wv = P.w + size_t(fl) * KD * Nmax;
        const cx<T>* u = s_uu + fl * Nmax;
        pidx[fl] = -1;
        for (int p = tid; p < N; p += NT) {
            cx<T> wold[KD];
#pragma unroll
            for (int j = 0; j < KD; ++j) wold[j] = j < np ? wv[j * Nmax + p] : cx<T>{T(0), T(0)};
            cx<T> acc;
            if (!full) {
                acc = col_dot<T>(A, N, p, u);
            } else {
                acc = {T(0), T(0)};
                cx<T> nw[KD];
#pragma unroll
                for (int j = 0; j < KD; ++j) nw[j] = {-wold[j].x, -wold[j].y};
                int f = 0;
                for (; f + 8 <= N; f += 8) {   // 8 loads in flight, then update and store
                    cx<T> a[8];
#pragma unroll
                    for (int q = 0; q < 8; ++q) a[q] = A[size_t(f + q) * N + p];
#pragma unroll
                    for (int q = 0; q < 8; ++q) {
                        cmac(acc, a[q], u[f + q]);
#pragma unroll
                        for (int j = 0; j < KD; ++j) cmac(a[q], nw[j], rr[j * Nmax + f + q]);
                        A[size_t(f + q) * N + p] = a[q];
                    }
                }
                for (; f < N; ++f) {
                    cx<T> a = A[size_t(f) * N + p];
                    cmac(acc, a, u[f]);
#pragma unroll
                    for (int j = 0; j < KD; ++j) cmac(a, nw[j], rr[j * Nmax + f]);
                    A[size_t(f) * N + p] = a;
                }
            }
#pragma unroll
            for (int j = 0; j < KD; ++j)
                if (j < np) cmac(acc, cx<T>{-wold[j].x, -wold[j].y}, sj[fl * KD + j]);
            if (p == c) acc.x -= T(1);
            wnew[fl] = acc;
            pidx[fl] = p;
        }
    }
    __syncthreads();   // every read of the old pairs is done
#pragma unroll
    for (int fl = 0; fl < 2; ++fl) {
        const int N = fl ? N1 : N0;
        const cx<T> inv = fl ? id : iu;
        for (int f = tid; f < N; f += NT) P.rr[(fl * KD + slot) * Nmax + f] = s_row[fl * Nmax + f] * inv;
        if (pidx[fl] >= 0) P.w[(fl * KD + slot) * Nmax + pidx[fl]] = wnew[fl];
    }
    P.n = slot + 1;
    __syncthreads();
}

template <typename T, int NT, int KD>
__global__ void __launch_bounds__(NT, 768 / NT) k_walk_gs(DevJob J, uint64_t nsteps, uint64_t s0, uint64_t meas, int mask,
                                                int inkernel_reinv, int measure_first)
{
    extern __shared__ __align__(16) char smem[];
    constexpr int NW = NT / 32;
    const int w = blockIdx.x;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (w >= J.W || J.status[w] != GV_OK) return;
    const bool forced = J.forced_walker >= 0;
    if (forced && w != J.forced_walker) return;
    const int Ns = J.Ns, Nmax = J.Nmax, L = J.L, Nk = J.Nk;
    const int N0 = J.N[0], N1 = J.N[1];
    const WalkLayout lay = walk_layout<T, NT, KD>(Ns, Nmax, (mask & GV_MEAS_PROJHEIS) != 0, inkernel_reinv != 0);
    Pending<T, KD> P = {reinterpret_cast<cx<T>*>(smem + lay.pend),
                        reinterpret_cast<cx<T>*>(smem + lay.pend) + 2 * KD * Nmax, 0};
    int16_t* s_fock = reinterpret_cast<int16_t*>(smem + lay.fock);
    int16_t* s_part = reinterpret_cast<int16_t*>(smem + lay.part);
    int16_t* s_nbr = reinterpret_cast<int16_t*>(smem + lay.nbr);
    cx<T>* s_coef = reinterpret_cast<cx<T>*>(smem + lay.coef);
    cx<T>* s_uu = reinterpret_cast<cx<T>*>(smem + lay.uu);
    cx<T>* s_row = reinterpret_cast<cx<T>*>(smem + lay.row);
    cx<T>* s_rr = reinterpret_cast<cx<T>*>(smem + lay.rr);
    double* s_red = reinterpret_cast<double*>(smem + lay.red);
    cx<T>* s_rq = reinterpret_cast<cx<T>*>(smem + lay.rdn);

    for (int i = tid; i < 2 * Ns; i += NT) s_fock[i] = J.fock[size_t(w) * 2 * Ns + i];
    for (int i = tid; i < 2 * Nmax; i += NT) s_part[i] = J.part[size_t(w) * 2 * Nmax + i];
    for (int i = tid; i < 4 * Ns; i += NT) s_nbr[i] = int16_t(J.nbr[i]);
    {
        const cx<T>* cg = Tab<T>::coef(J) + size_t(w) * 4 * Ns;   // [fl][sub][orbital]
        for (int i = tid; i < 4 * Nmax; i += NT) {
            const int fl = i / (2 * Nmax), sub = (i / Nmax) & 1, f = i % Nmax;
            s_coef[i] = cg[(size_t(fl) * 2 + sub) * Ns + 2 * f];
        }
    }
    __syncthreads();

    const cx<T>* phase = Tab<T>::phase(J);
    cx<T>* A0 = ai_ptr<T>(J, 0, w);
    cx<T>* A1 = ai_ptr<T>(J, 1, w);
    const uint32_t wid = J.walker_base + uint32_t(w);
    uint64_t k = J.rng_next[w];
    unsigned long long c_acc = 0, c_noop = 0, c_rej = 0, c_reinv = 0;
    int since = J.since_reinv[w];
    cx<double> am = J.amp_m[w];
    int ae = J.amp_e[w];
    int status = GV_OK;
    int rbuf = 0;
    const WalkCtx<T> C = {&J, w, Ns, Nmax, L, Nk, N0, N1, s_fock, s_part, s_nbr, s_coef, s_rq, s_red + 2 * NW * 4,
                          phase, A0, A1};
    if (measure_first && mask) measure_now<T, NT>(C, mask);

    for (uint64_t s = 0; s < nsteps; ++s, k += 4) {
        uint32_t x[4], y[4];
        philox_call(J.seed, wid, 0, k >> 1, x);
        philox_call(J.seed, wid, 0, (k >> 1) + 1, y);
        // u1 -> vertex, u2 -> neighbour slot, u3 unused, u4 -> accept test; the
        // vertex and slot are computed in integers, bit-identical to
        // size_t(n * uniform()) (LatticeStepper.cpp:45-47).
        const uint64_t m4 = u52(y[2], y[3]);
        int v1 = scaled_floor(uint32_t(Ns), u52(x[0], x[1]));
        int v2 = s_nbr[v1 * 4 + int(u52(x[2], x[3]) >> 50)];
        if (forced) { v1 = J.forced_v1; v2 = J.forced_v2; }
        const int f1 = s_fock[v1] >= 0 ? 0 : 1;
        const int f2 = s_fock[v2] >= 0 ? 0 : 1;
        int kind = 0, accepted;
        T ratio = T(1);
        if (f1 == f2) {
            accepted = 1;   // m_weight / m_state_weight = 1, u4 < 1 (MetroMC.cpp:41)
            ++c_noop;
        } else {
            kind = 1;
            const int upf = (f1 == 0) ? v1 : v2, upt = (f1 == 0) ? v2 : v1;
            const int dnf = upt, dnt = upf;
            const int cu = s_fock[upf], cd = s_fock[Ns + dnf];
            cx<T> au = {T(0), T(0)}, ad = {T(0), T(0)};
            for (int f = tid; f < N0; f += NT) {
                cx<T> a = A0[size_t(f) * N0 + cu];
                for (int j = 0; j < P.n; ++j) {   // current row c: stored row minus pending pairs
                    const cx<T> wj = P.w[j * Nmax + cu];
                    cmac(a, cx<T>{-wj.x, -wj.y}, P.rr[j * Nmax + f]);
                }
                const cx<T> u = phi_row<T>(phase, s_coef, Nk, Nmax, L, upt, f);
                s_row[f] = a;
                s_uu[f] = u;
                cmac(au, a, u);
            }
            for (int f = tid; f < N1; f += NT) {
                cx<T> a = A1[size_t(f) * N1 + cd];
                for (int j = 0; j < P.n; ++j) {
                    const cx<T> wj = P.w[(KD + j) * Nmax + cd];
                    cmac(a, cx<T>{-wj.x, -wj.y}, P.rr[(KD + j) * Nmax + f]);
                }
                const cx<T> u = phi_row<T>(phase, s_coef + 2 * Nmax, Nk, Nmax, L, dnt, f);
                s_row[Nmax + f] = a;
                s_uu[Nmax + f] = u;
                cmac(ad, a, u);
            }
            au = warp_sum(au);
            ad = warp_sum(ad);
            T* rb = reinterpret_cast<T*>(s_red) + rbuf * NW * 4;
            rbuf ^= 1;
            if (lane == 0) { rb[warp * 4 + 0] = au.x; rb[warp * 4 + 1] = au.y; rb[warp * 4 + 2] = ad.x; rb[warp * 4 + 3] = ad.y; }
            __syncthreads();
            cx<T> ru = {T(0), T(0)}, rd = {T(0), T(0)};
            for (int q = 0; q < NW; ++q) {
                ru.x += rb[q * 4 + 0]; ru.y += rb[q * 4 + 1];
                rd.x += rb[q * 4 + 2]; rd.y += rb[q * 4 + 3];
            }
            ratio = Accept<T>::ratio(ru, rd);
            if (!isfinite(ratio)) { status = GV_ERR_NAN; break; }
            // MetroMC::YesNo (MetroMC.cpp:41): ratio > 1 draws u4 < 1, always true here
            accepted = forced ? J.forced_accept : (ratio > T(1) ? 1 : (Accept<T>::uniform(m4) < ratio));
            if (!accepted) {
                ++c_rej;
            } else {
                if (norm2(ru) < T(1e-9) || norm2(rd) < T(1e-9)) { status = GV_ERR_SINGULAR; break; }
                const cx<T> iu = cinv(ru), id = cinv(rd);
                if constexpr (KD == 0) {
                    for (int f = tid; f < N0; f += NT) s_rr[f] = s_row[f] * iu;
                    for (int f = tid; f < N1; f += NT) s_rr[Nmax + f] = s_row[Nmax + f] * id;
                    __syncthreads();
                    // Per particle column p (one owner thread): w_p = (A^-1 u)_p - [p == c],
                    // then column update with the old row c of A^-1 divided by r.
                    for (int p = tid; p < N0; p += NT) {
                        cx<T> wp = col_dot<T>(A0, N0, p, s_uu);
                        if (p == cu) wp.x -= T(1);
                        col_update<T>(A0, N0, p, wp, s_rr);
                    }
                    for (int p = tid; p < N1; p += NT) {
                        cx<T> wp = col_dot<T>(A1, N1, p, s_uu + Nmax);
                        if (p == cd) wp.x -= T(1);
                        col_update<T>(A1, N1, p, wp, s_rr + Nmax);
                    }
                    __syncthreads();
                } else {
                    accept_delayed<T, NT, KD>(P, A0, A1, N0, N1, Nmax, cu, cd, iu, id, s_row, s_uu,
                                              reinterpret_cast<T*>(smem + lay.redk));
                }
                if (tid == 0) {
                    s_fock[upt] = int16_t(cu); s_fock[upf] = -1; s_part[cu] = int16_t(upt);
                    s_fock[Ns + dnt] = int16_t(cd); s_fock[Ns + dnf] = -1; s_part[Nmax + cd] = int16_t(dnt);
                }
                if (tid == 0) {   // the amplitude lives in thread 0 (FP64, once per accept)
                    am = am * (to_d(ru) * to_d(rd));
                    amp_normalise(am, ae);
                }
                ++c_acc;
                ++since;
                __syncthreads();
                if (inkernel_reinv && J.reinv_every > 0 && since >= J.reinv_every) {
                    flush_pending<T, NT, KD>(P, A0, A1, N0, N1, Nmax);
                    char* gp = smem + lay.gj;
                    GJSmem G = carve_gj<NT>(gp, Nmax);
                    cx<double>* M = J.scratch64 + size_t(w) * Nmax * Nmax;
                    const int st = reinvert_walker<T, NT>(J, w, M, G, s_part);
                    if (st != GV_OK) { status = st; break; }
                    am = J.amp_m[w];
                    ae = J.amp_e[w];
                    since = 0;
                    ++c_reinv;
                }
            }
        }
        if (J.trace && w == J.trace_walker && tid == 0) {
            gv_trace t;
            t.v1 = v1; t.v2 = v2; t.kind = kind; t.accepted = accepted; t.khop = kind ? 0 : -1; t.pad = 0;
            t.ratio = double(ratio); t.u4 = u01(y[2], y[3]);
            J.trace[s] = t;
        }
        if (forced && !J.forced_accept) return;   // evaluation only: nothing was changed, nothing to write
        const uint64_t gs = s0 + s;
        if (meas && (meas == 1 || gs % meas == 0) && mask) {
            flush_pending<T, NT, KD>(P, A0, A1, N0, N1, Nmax);
            measure_now<T, NT>(C, mask);
        }
    }
    flush_pending<T, NT, KD>(P, A0, A1, N0, N1, Nmax);
    __syncthreads();
    for (int i = tid; i < 2 * Ns; i += NT) J.fock[size_t(w) * 2 * Ns + i] = s_fock[i];
    for (int i = tid; i < 2 * Nmax; i += NT) J.part[size_t(w) * 2 * Nmax + i] = s_part[i];
    if (tid == 0) {
        if (!forced) J.rng_next[w] = k;   // single-walker stepping draws its uniforms itself
        unsigned long long* c = J.counts + size_t(w) * 5;
        c[0] += c_acc + c_noop + c_rej;
        c[1] += c_acc;
        c[2] += c_noop;
        c[3] += c_rej;
        c[4] += c_reinv;
        J.since_reinv[w] = since;
        J.amp_m[w] = am;
        J.amp_e[w] = ae;
        J.status[w] = status;
    }
}

// StagMagnTrack / OverlapTrack (StagMagnTrack.cpp:21-50; OverlapTrack.cpp:26-29):
// one warp per walker appends the staggered magnetisation and log10 of the
// stepper weight (|Amp|^2, times sigma = sum_k |q_k|^2 / |Amp|^2 in the
// exciton channel) to the walker's tracks.
__global__ void k_tracks(DevJob J, int mask)
{
    const int w = int(blockIdx.x) * (blockDim.x / 32) + int(threadIdx.x / 32), lane = threadIdx.x & 31;
    if (w >= J.W || J.status[w] != GV_OK) return;
    const int n = J.track_n[w];
    if (n >= J.track_cap) return;
    const size_t at = size_t(w) * J.track_cap + n;
    if (mask & GV_MEAS_STAGMAGN_TRACK) {
        const int16_t* fock = J.fock + size_t(w) * 2 * J.Ns;
        int m = 0;
        for (int v = lane; v < J.Ns; v += 32) {
            const int sg = (((v % J.L) + (v / J.L)) & 1) ? -1 : 1;
            m += sg * (fock[v] >= 0 ? 1 : -1);
        }
#pragma unroll
        for (int o = 16; o; o >>= 1) m += __shfl_xor_sync(0xffffffffu, m, o);
        if (lane == 0) J.track_sm[at] = double(m) / double(J.Ns);
    }
    if (lane == 0) {
        if (mask & GV_MEAS_OVERLAP_TRACK) {
            const cx<double> a = J.amp_m[w];
            const double mag = hypot(a.x, a.y);
            double lw = mag > 0.0 ? 2.0 * (log10(mag) + double(J.amp_e[w]) * 0.30102999566398119521) : -INFINITY;
            if (J.channel != GV_CH_GROUNDSTATE) lw += log10(J.sigma[w]);
            J.track_lw[at] = lw;
        }
        J.track_n[w] = n + 1;
    }
}

// Ratio of moving particle c of flavour fl to site d (one warp, lanes over
// rows); row f's orbital has phase column pcol_fl[f] and coefficients
// coef_fl[sub][f].
template <typename T>
__device__ __forceinline__ cx<T> warp_ratio(const DevJob& J, const cx<T>* A, const cx<T>* phase,
                                            const cx<T>* coef_fl, const int16_t* pcol_fl, int N, int c, int d)
{
    const int lane = threadIdx.x & 31;
    const int sub = sublattice(d, J.L);
    cx<T> acc = {T(0), T(0)};
    for (int f = lane; f < N; f += 32)
        cmac(acc, A[size_t(f) * N + c], cmul_rn(phase[size_t(d) * J.Nk + pcol_fl[f]], coef_fl[sub * J.Nmax + f]));
    return warp_sum(acc);
}

// StatSpinStruct (StatSpinStruct.cpp:16-135), two flavours, accumulated in
// compact form: for every antiparallel pair (flavour-0 particle c at site i,
// flavour-1 particle q at site j), one warp per pair,
//     T[i][j]   += r_up(c -> j) r_dn(q -> i)   (the reference's conj(amp) swamp / w)
//     Aud[i][j] += 1
// (T complex, Aud real, both Ns x Ns, job-wide).  szz, s+- and s-+ follow
// from them and the occupation counts they imply (gv_job_read_statspin).  In
// the exciton channel the swap keeps the channel state and w is the weight
// over all states, so the ratio is divided by sigma = w / |Amp|^2.
template <typename T, int NT>
__global__ void __launch_bounds__(NT) k_statspin(DevJob J)
{
    const int w = blockIdx.x;
    if (w >= J.W || J.status[w] != GV_OK) return;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    constexpr int NW = NT / 32;
    const int Ns = J.Ns, Nmax = J.Nmax, N0 = J.N[0], N1 = J.N[1];
    const int16_t* part = J.part + size_t(w) * 2 * Nmax;
    const cx<T>* phase = Tab<T>::phase(J);
    const cx<T>* cg = Tab<T>::coef(J) + size_t(w) * 4 * Ns;
    extern __shared__ __align__(16) char smem[];
    cx<T>* coef = reinterpret_cast<cx<T>*>(smem);
    int16_t* pcol = reinterpret_cast<int16_t*>(coef + 4 * Nmax);
    for (int i = tid; i < 4 * Nmax; i += NT) {
        const int fl = i / (2 * Nmax), sub = (i / Nmax) & 1, f = i % Nmax;
        const int o = f < J.N[fl] ? row_orbital(J, nullptr, w, fl, f) : 0;
        coef[i] = cg[(size_t(fl) * 2 + sub) * Ns + o];
        if (!sub) pcol[fl * Nmax + f] = int16_t(o >> 1);
    }
    __syncthreads();
    const bool scaled = J.channel != GV_CH_GROUNDSTATE;
    const double inv_sigma = scaled ? 1.0 / J.sigma[w] : 1.0;
    const cx<T>* A0 = ai_ptr<T>(J, 0, w);
    const cx<T>* A1 = ai_ptr<T>(J, 1, w);
    double* Tsum = J.ss;
    double* Aud = J.ss + 2 * size_t(Ns) * Ns;
    for (int idx = warp; idx < N0 * N1; idx += NW) {
        const int c = idx / N1, q = idx % N1;
        const int si = part[c], sj = part[Nmax + q];
        const cx<T> ru = warp_ratio<T>(J, A0, phase, coef, pcol, N0, c, sj);
        const cx<T> rd = warp_ratio<T>(J, A1, phase, coef + 2 * Nmax, pcol + Nmax, N1, q, si);
        if (lane == 0) {
            cx<double> r = to_d(ru) * to_d(rd);
            if (scaled) r = r * inv_sigma;
            const size_t ij = size_t(si) * Ns + sj;
            atomicAdd(&Tsum[2 * ij], r.x);
            atomicAdd(&Tsum[2 * ij + 1], r.y);
            atomicAdd(&Aud[ij], 1.0);
        }
    }
    if (tid == 0) atomicAdd(J.ss_n, w == 0 ? 1 : 0);
}

// s + c += a x with a = ah + al (double-float) and x exact: exact product
// (Dekker, via FMA) and compensated sum (Knuth's two-sum), every operation
// explicitly rounded so that nothing is contracted or reassociated.
__device__ __forceinline__ void ff_madd(float& s, float& c, float ah, float al, float x)
{
    const float p = __fmul_rn(ah, x);
    const float e = __fmaf_rn(ah, x, -p);
    const float t = __fadd_rn(s, p);
    const float bb = __fsub_rn(t, s);
    const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bb)), __fsub_rn(p, bb));
    s = t;
    c = __fadd_rn(c, __fadd_rn(err, __fadd_rn(e, __fmul_rn(al, x))));
}

// s + c += s2 + c2 (two double-float numbers)
__device__ __forceinline__ void ff_add(float& s, float& c, float s2, float c2)
{
    const float t = __fadd_rn(s, s2);
    const float bb = __fsub_rn(t, s);
    const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bb)), __fsub_rn(s2, bb));
    s = t;
    c = __fadd_rn(c, __fadd_rn(err, c2));
}

__device__ __forceinline__ void ff_cmac(cx<float>& s, cx<float>& c, cx<float> ah, cx<float> al, cx<float> x)
{
    ff_madd(s.x, c.x, ah.x, al.x, x.x);
    ff_madd(s.x, c.x, -ah.y, -al.y, x.y);
    ff_madd(s.y, c.y, ah.x, al.x, x.y);
    ff_madd(s.y, c.y, ah.y, al.y, x.x);
}

// Drift-checked re-inversion (deferred policy).  For every walker whose
// accepted-exchange count since the last check reached reinv_every, estimate
// ||A A^-1 - I||_max to FP64 accuracy on 8 rows f of the residual (rows rotate
// from check to check): (A A^-1)(f, g) = sum_p phi_{2f}(x_p) (A^-1)(p, g),
// with A rebuilt in FP64 from the orbital tables; for an FP32-stored inverse
// the sums run in double-float arithmetic on the FP32 pipe (GB300's FP64 rate
// is 1/64 of its FP32 rate).  Walkers above the threshold (or
// all of them when threshold < 0) get the FP64 Gauss-Jordan re-inversion.
template <typename T, int NT>
__global__ void __launch_bounds__(NT, 2) k_check_reinvert(DevJob J, double threshold, int m_in_smem)
{
    extern __shared__ __align__(16) char smem[];
    constexpr int NR = 8;
    constexpr int NW = NT / 32;
    const int w = blockIdx.x;
    if (w >= J.W || J.status[w] != GV_OK || J.reinv_every <= 0 || J.since_reinv[w] < J.reinv_every) return;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int Nmax = J.Nmax, Ns = J.Ns;
    cx<double>* arow = reinterpret_cast<cx<double>*>(smem);             // 2 * NR * Nmax
    double* red = reinterpret_cast<double*>(arow + 2 * NR * Nmax);      // NW
    char* gp = reinterpret_cast<char*>(red + NW + 2);
    gp = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(gp) + 15) & ~uintptr_t(15));
    double drift = 0.0;
    if (threshold >= 0.0) {
        const unsigned long long nchk = J.counts[size_t(w) * 5 + 4] + J.checks[w];
        auto sampled = [&](int i, int N) { return int((nchk * NR + size_t(i) * (N / NR) + i) % N); };
        // the sampled rows of A of both flavours, FP64
        for (int fl = 0; fl < 2; ++fl) {
            const int N = J.N[fl];
            const int16_t* part = J.part + (size_t(w) * 2 + fl) * Nmax;
            const cx<double>* coef = J.coef64 + (size_t(w) * 2 + fl) * 2 * Ns;
            for (int idx = tid; idx < NR * N; idx += NT) {
                const int i = idx / N, p = idx % N;
                const int site = part[p];
                const int o = row_orbital(J, nullptr, w, fl, sampled(i, N));
                const cx<double> v = cmul_rn(J.phase64[size_t(site) * J.Nk + (o >> 1)],
                                             coef[size_t(sublattice(site, J.L)) * Ns + o]);
                if constexpr (sizeof(T) == 4) {   // hi + lo floats, same bytes as one FP64 complex
                    cx<float>* ahi = reinterpret_cast<cx<float>*>(arow + fl * NR * Nmax);
                    const cx<float> h = {float(v.x), float(v.y)};
                    ahi[i * Nmax + p] = h;
                    ahi[(NR + i) * Nmax + p] = cx<float>{float(v.x - double(h.x)), float(v.y - double(h.y))};
                } else {
                    arow[(fl * NR + i) * Nmax + p] = v;
                }
            }
        }
        __syncthreads();
        if constexpr (sizeof(T) == 4) {
            // FP32-stored inverse: the residual (A A^-1)(i, g) = sum_p A(i, p) AiT[g][p]
            // in double-float arithmetic on the FP32 pipe (A's FP64 entries split into
            // hi + lo floats, exact products, compensated sums), one thread per row g
            // of AiT of either flavour, so that no lane sums are needed
            for (int idx = tid; idx < J.N[0] + J.N[1]; idx += NT) {
                const int fl = idx < J.N[0] ? 0 : 1, g = fl ? idx - J.N[0] : idx, N = J.N[fl];
                const cx<float>* ahi = reinterpret_cast<const cx<float>*>(arow + fl * NR * Nmax);
                const cx<float>* alo = ahi + NR * Nmax;
                const cx<float>* Ag = reinterpret_cast<const cx<float>*>(ai_ptr<T>(J, fl, w)) + size_t(g) * N;
                cx<float> sm[NR], cm[NR];
#pragma unroll
                for (int i = 0; i < NR; ++i) { sm[i] = {0.f, 0.f}; cm[i] = {0.f, 0.f}; }
                for (int p = 0; p < N; ++p) {
                    const cx<float> x = Ag[p];
#pragma unroll
                    for (int i = 0; i < NR; ++i) ff_cmac(sm[i], cm[i], ahi[i * Nmax + p], alo[i * Nmax + p], x);
                }
#pragma unroll
                for (int i = 0; i < NR; ++i) {
                    cx<double> v = {double(sm[i].x) + double(cm[i].x), double(sm[i].y) + double(cm[i].y)};
                    if (sampled(i, N) == g) v.x -= 1.0;
                    drift = fmax(drift, fmax(fabs(v.x), fabs(v.y)));
                }
            }
        } else {
            for (int fl = 0; fl < 2; ++fl) {
                const int N = J.N[fl];
                const cx<T>* A = ai_ptr<T>(J, fl, w);
                for (int g = warp; g < N; g += NW) {
                    cx<double> acc[NR];
#pragma unroll
                    for (int i = 0; i < NR; ++i) acc[i] = {0.0, 0.0};
                    for (int p = lane; p < N; p += 32) {
                        const cx<double> x = to_d(A[size_t(g) * N + p]);
#pragma unroll
                        for (int i = 0; i < NR; ++i) cmac(acc[i], arow[(fl * NR + i) * Nmax + p], x);
                    }
#pragma unroll
                    for (int i = 0; i < NR; ++i) {
                        cx<double> v = warp_sum(acc[i]);
                        if (sampled(i, N) == g) v.x -= 1.0;
                        drift = fmax(drift, fmax(fabs(v.x), fabs(v.y)));
                    }
                }
            }
        }
#pragma unroll
        for (int o = 16; o; o >>= 1) drift = fmax(drift, __shfl_xor_sync(0xffffffffu, drift, o));
        if (lane == 0) red[warp] = drift;
        __syncthreads();
        drift = 0.0;
        for (int q = 0; q < NW; ++q) drift = fmax(drift, red[q]);
        __syncthreads();
    }
    const bool redo = threshold < 0.0 || drift > threshold;
    if (redo) {
        GJSmem S = carve_gj<NT>(gp, Nmax);
        // the working matrix after the GJ scratch when the launch provides it (as k_invert)
        cx<double>* M = m_in_smem ? reinterpret_cast<cx<double>*>(gp) : J.scratch64 + size_t(w) * Nmax * Nmax;
        const int st = reinvert_walker<T, NT>(J, w, M, S, nullptr);
        if (J.channel == GV_CH_TRANS && st == GV_OK) trans_rebuild<T, NT>(J, w, nullptr, J.cur[w]);
        if (J.channel == GV_CH_LONG && st == GV_OK) long_rebuild<T, NT>(J, w, nullptr);
        if (tid == 0) { J.status[w] = st; J.counts[size_t(w) * 5 + 4] += 1; }
    } else if (tid == 0) {
        J.checks[w] += 1;
    }
    if (tid == 0) {
        J.since_reinv[w] = 0;
        J.drift_seen[w] = fmax(J.drift_seen[w], drift);
    }
}

__host__ __device__ inline size_t check_smem_bytes(int Nmax, int NT)
{
    return sizeof(cx<double>) * 2 * 8 * Nmax + sizeof(double) * (NT / 32 + 2) + 16 + gj_smem_bytes(Nmax, NT) + 16;
}

// VirtUpdate-style ratios for explicit hop sets of one walker.
template <typename T>
__global__ void k_virt_update(DevJob J, int w, int nset, const int32_t* hops, double* out)
{
    const int lane = threadIdx.x & 31;
    const int set = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
    if (set >= nset) return;
    const int Ns = J.Ns;
    const int16_t* fock = J.fock + size_t(w) * 2 * Ns;
    const cx<T>* cg = Tab<T>::coef(J) + size_t(w) * 4 * Ns;
    const cx<T>* phase = Tab<T>::phase(J);
    cx<double> r = {1.0, 0.0};
    for (int fl = 0; fl < 2; ++fl) {
        const int from = hops[4 * set + 2 * fl], to = hops[4 * set + 2 * fl + 1];
        if (from < 0) continue;
        const int c = fock[fl * Ns + from];
        if (c < 0) { r = cx<double>{nan(""), nan("")}; break; }   // no particle of this flavour there
        const int N = J.N[fl];
        const cx<T>* A = ai_ptr<T>(J, fl, w);
        cx<T> acc = {T(0), T(0)};
        const int sub = sublattice(to, J.L);
        for (int f = lane; f < N; f += 32)
            cmac(acc, A[size_t(f) * N + c], cmul_rn(phase[size_t(to) * J.Nk + f], cg[(size_t(fl) * 2 + sub) * Ns + 2 * f]));
        acc = warp_sum(acc);
        r = r * to_d(acc);
    }
    if (lane == 0) { out[2 * set] = r.x; out[2 * set + 1] = r.y; }
}

// max |(A A^-1 - I)_{f g}| per walker/flavour in FP64.
template <typename T, int NT>
__global__ void __launch_bounds__(NT) k_drift(DevJob J, double* out)
{
    const int w = blockIdx.x, fl = blockIdx.y;
    const int N = J.N[fl], Ns = J.Ns;
    const int16_t* part = J.part + (size_t(w) * 2 + fl) * J.Nmax;
    const cx<double>* coef = J.coef64 + (size_t(w) * 2 + fl) * 2 * Ns;
    const cx<T>* A = ai_ptr<T>(J, fl, w);
    double mx = 0.0;
    for (int idx = threadIdx.x; idx < N * N; idx += NT) {
        const int f = idx / N, g = idx % N;
        cx<double> s = {0.0, 0.0};
        for (int pr = 0; pr < N; ++pr) {
            const int site = part[pr];
            const int o = row_orbital(J, nullptr, w, fl, f);
            const cx<double> a = cmul_rn(J.phase64[size_t(site) * J.Nk + (o >> 1)], coef[size_t(sublattice(site, J.L)) * Ns + o]);
            cmac(s, a, to_d(A[size_t(g) * N + pr]));
        }
        if (f == g) s.x -= 1.0;
        mx = fmax(mx, fmax(fabs(s.x), fabs(s.y)));
    }
    __shared__ double red[NT / 32];
#pragma unroll
    for (int o = 16; o; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
        double m = 0;
        for (int q = 0; q < NT / 32; ++q) m = fmax(m, red[q]);
        out[w * 2 + fl] = m;
    }
}

}  // namespace
}  // namespace gv
