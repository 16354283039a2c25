// GB300 engine for the gpvmc Metropolis sampling path: kernels and the C ABI
// declared in include/gpvmc_gb300.h.
//
// Layout in HBM, per job (W walkers, flavour fl in {0: flavour-0 "up", 1}):
//   phase   [Ns][Nk]            sqrt(2) e^{i k.r}, shared by all walkers (L2-resident)
//   coef    [W][fl][sub][Ns]    U_k / V_k of every orbital for the walker's (phi, neel)
//   Ai[fl]  [W][N][N]           inverse Slater matrix, row-major (particle p, row f):
//                               Ai[p][f] = (A^-1)(p, f), A(f, p) = phi_{orb f}(site of p)
//   fock    [W][fl][Ns]  int16  particle at a site or -1;  part [W][fl][N] site of a particle
//   amp     [W]                 complex mantissa + base-2 exponent of Amp()
// phi_o(s) is never stored per walker: it is phase[s][o/2] * coef[sub(s)][o]
// assembled in registers, so a proposal reads one inverse row per flavour
// from HBM and the phase column from L2.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "device.cuh"
#include "model.hpp"

using namespace gv;

namespace {

// ------------------------------------------------------------------------
// Small device helpers

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

// ------------------------------------------------------------------------
// FP64 Gauss-Jordan inversion with partial (row) pivoting on max |re|+|im|,
// in place on M (N x N row-major, global scratch).  Pivots equal those of
// LAPACK zgetrf, so det = prod(pivots) * (-1)^swaps as in linalg::DetInv
// (linalg.cpp:9-44).  Returns false if a pivot column is exactly zero.
template <int NT>
__device__ bool gj_invert(cx<double>* M, int N, cx<double>* rowk, cx<double>* fcol, int* perm,
                          double* redv, int* redi, cx<double>& det_m, int& det_e)
{
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    constexpr int NW = NT / 32;
    cx<double> dm = {1.0, 0.0};
    int de = 0;
    for (int k = 0; k < N; ++k) {
        double best = -1.0;
        int bi = N;
        for (int i = k + tid; i < N; i += NT) {
            cx<double> v = M[size_t(i) * N + k];
            double a = fabs(v.x) + fabs(v.y);
            if (a > best) { best = a; bi = i; }
        }
#pragma unroll
        for (int o = 16; o; o >>= 1) {
            double ob = __shfl_xor_sync(0xffffffffu, best, o);
            int oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
        }
        if (lane == 0) { redv[warp] = best; redi[warp] = bi; }
        __syncthreads();
        best = redv[0];
        bi = redi[0];
        for (int q = 1; q < NW; ++q)
            if (redv[q] > best || (redv[q] == best && redi[q] < bi)) { best = redv[q]; bi = redi[q]; }
        if (!(best > 0.0)) return false;
        const int p = bi;
        if (p != k)
            for (int j = tid; j < N; j += NT) {
                cx<double> a = M[size_t(k) * N + j];
                M[size_t(k) * N + j] = M[size_t(p) * N + j];
                M[size_t(p) * N + j] = a;
            }
        __syncthreads();
        const cx<double> piv = M[size_t(k) * N + k];
        if (tid == 0) {
            perm[k] = p;
            dm = dm * piv;
            if (p != k) { dm.x = -dm.x; dm.y = -dm.y; }
            amp_normalise(dm, de);
        }
        const cx<double> inv = cinv(piv);
        for (int j = tid; j < N; j += NT) {
            cx<double> v = (j == k) ? cx<double>{1.0, 0.0} : M[size_t(k) * N + j];
            v = v * inv;
            rowk[j] = v;
        }
        for (int i = tid; i < N; i += NT) fcol[i] = (i == k) ? cx<double>{0.0, 0.0} : M[size_t(i) * N + k];
        __syncthreads();
        for (int j = tid; j < N; j += NT) M[size_t(k) * N + j] = rowk[j];
        for (int i = warp; i < N; i += NW) {
            if (i == k) continue;
            const cx<double> f = fcol[i];
            for (int j = lane; j < N; j += 32) {
                cx<double> v = (j == k) ? cx<double>{0.0, 0.0} : M[size_t(i) * N + j];
                cmac(v, cx<double>{-f.x, -f.y}, rowk[j]);
                M[size_t(i) * N + j] = v;
            }
        }
        __syncthreads();
    }
    for (int k = N - 1; k >= 0; --k) {
        const int p = perm[k];
        if (p != k)
            for (int i = tid; i < N; i += NT) {
                cx<double> a = M[size_t(i) * N + k];
                M[size_t(i) * N + k] = M[size_t(i) * N + p];
                M[size_t(i) * N + p] = a;
            }
        __syncthreads();
    }
    if (tid == 0) { det_m = dm; det_e = de; }
    return true;
}

// Shared-memory scratch used by gj_invert.
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

// SlaterDeterminant::Init for walker w (SlaterDeterminant.cpp:60-92): build
// A(f, r) = phi_{2f}(site of particle r) in FP64 (ground-state rows), invert,
// store Ai in T, amplitude = det_0 * det_1.  Returns a gv_status.
template <typename T, int NT>
__device__ int reinvert_walker(const DevJob& J, int w, cx<double>* M, const GJSmem& S,
                               const int16_t* part_s /* smem or null */)
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
            const int f = idx / N, r = idx % N;
            const int s = part[r];
            const int sub = sublattice(s, J.L);
            M[idx] = cmul_rn(J.phase64[size_t(s) * J.Nk + f], coef[size_t(sub) * J.Ns + 2 * f]);
        }
        __syncthreads();
        cx<double> dm;
        int de;
        bool ok = gj_invert<NT>(M, N, S.rowk, S.fcol, S.perm, S.redv, S.redi, dm, de);
        if (tid == 0) { S.detm[0] = dm; S.dete[0] = de; S.flag[0] = ok; }
        __syncthreads();
        ok = S.flag[0];
        dm = S.detm[0];
        de = S.dete[0];
        __syncthreads();
        // reference: singular if |det|^2 < 1e-9, amplitude zero if exponent10 < -8
        double l10 = ok ? (log10(sqrt(norm2(dm))) + de * 0.30102999566398119521) : -1e300;
        if (!ok || 2.0 * l10 < -9.0 || floor(l10) < -8.0) status = GV_ERR_SINGULAR;
        cx<T>* out = ai_ptr<T>(J, fl, w);
        for (int idx = tid; idx < N * N; idx += NT) {
            cx<double> v = M[idx];
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
    return status;
}

template <int NT>
__device__ GJSmem carve_gj(char*& p, int Nmax)
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

template <typename T, int NT>
__global__ void __launch_bounds__(NT) k_invert(DevJob J, int w0, int nw)
{
    extern __shared__ __align__(16) char smem[];
    const int w = w0 + blockIdx.x;
    if (blockIdx.x >= nw || w >= J.W) return;
    char* p = smem;
    GJSmem S = carve_gj<NT>(p, J.Nmax);
    cx<double>* M = J.scratch64 + size_t(blockIdx.x) * J.Nmax * J.Nmax;
    int st = reinvert_walker<T, NT>(J, w, M, S, nullptr);
    if (threadIdx.x == 0) J.status[w] = st;
}

// ------------------------------------------------------------------------
// Metropolis walk, ground-state channel.  One CTA per walker; the walker's
// occupancy, coefficients and work vectors live in shared memory, its
// inverses in HBM.  Each step follows MetroMC::Step (MetroMC.cpp:90-103):
// 4 uniforms (vertex, neighbour, internal state, accept), a no-op for equal
// flavours, otherwise the two determinant ratios
//   r_fl = sum_f Ai_fl[c][f] phi_{2f}(d)       (linalg.cpp:297-303 / 146)
// and, on acceptance, the Sherman-Morrison update of both inverses
//   Ai <- Ai - (Ai u - e_c)(e_c^T Ai)/r        (linalg.cpp:402-573, rc=1 rr=0).
template <typename T, int NT>
struct WalkSmem {
    int16_t* fock;   // 2*Ns
    int16_t* part;   // 2*Nmax
    int32_t* nbr;    // 4*Ns
    cx<T>* coef;     // 2 fl * 2 sub * Nmax   (row f -> orbital 2f)
    cx<T>* uu;       // 2*Nmax
    cx<T>* row;      // 2*Nmax
    cx<T>* wv;       // 2*Nmax
    double* red;     // 2 buffers * (NT/32) * 4
    double* redm;    // NT/32 * 4 (measurements)
};

template <typename T, int NT>
__host__ __device__ inline size_t walk_smem_bytes(int Ns, int Nmax)
{
    size_t b = 0;
    b += sizeof(int16_t) * (2 * Ns + 2 * Nmax);
    b = (b + 15) & ~size_t(15);
    b += sizeof(int32_t) * 4 * Ns;
    b = (b + 15) & ~size_t(15);
    b += sizeof(cx<T>) * (4 * Nmax + 6 * Nmax);
    b += sizeof(double) * (2 * (NT / 32) * 4 + (NT / 32) * 4);
    b = (b + 15) & ~size_t(15);
    b += gj_smem_bytes(Nmax, NT) + 16;
    return b;
}

template <typename T>
__device__ __forceinline__ cx<T> phi_at(const cx<T>* phase, const cx<T>* coef_fl, int Nk, int Nmax, int L, int s, int f)
{
    // GS row f <-> orbital 2f: phase index f, coefficient of orbital 2f
    const int sub = sublattice(s, L);
    return cmul_rn(phase[size_t(s) * Nk + f], coef_fl[sub * Nmax + f]);
}

// Ratio of moving particle c of flavour fl to site d: one warp.
template <typename T>
__device__ __forceinline__ cx<T> warp_ratio(const DevJob& J, const cx<T>* Ai, const cx<T>* phase,
                                            const cx<T>* coef_fl, int N, int c, int d)
{
    const int lane = threadIdx.x & 31;
    cx<T> acc = {T(0), T(0)};
    const cx<T>* row = Ai + size_t(c) * N;
    for (int f = lane; f < N; f += 32) cmac(acc, row[f], phi_at<T>(phase, coef_fl, J.Nk, J.Nmax, J.L, d, f));
    return warp_sum(acc);
}

template <typename T, int NT>
__global__ void __launch_bounds__(NT) k_walk_gs(DevJob J, uint64_t nsteps, uint64_t s0, uint64_t meas, int mask)
{
    extern __shared__ __align__(16) char smem[];
    constexpr int NW = NT / 32;
    const int w = blockIdx.x;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (w >= J.W) return;
    if (J.status[w] != GV_OK) return;
    const int Ns = J.Ns, Nmax = J.Nmax, L = J.L;
    const int N0 = J.N[0], N1 = J.N[1];

    char* p = smem;
    WalkSmem<T, NT> S;
    S.fock = reinterpret_cast<int16_t*>(p); p += sizeof(int16_t) * 2 * Ns;
    S.part = reinterpret_cast<int16_t*>(p); p += sizeof(int16_t) * 2 * Nmax;
    p = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(p) + 15) & ~uintptr_t(15));
    S.nbr = reinterpret_cast<int32_t*>(p); p += sizeof(int32_t) * 4 * Ns;
    p = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(p) + 15) & ~uintptr_t(15));
    S.coef = reinterpret_cast<cx<T>*>(p); p += sizeof(cx<T>) * 4 * Nmax;
    S.uu = reinterpret_cast<cx<T>*>(p); p += sizeof(cx<T>) * 2 * Nmax;
    S.row = reinterpret_cast<cx<T>*>(p); p += sizeof(cx<T>) * 2 * Nmax;
    S.wv = reinterpret_cast<cx<T>*>(p); p += sizeof(cx<T>) * 2 * Nmax;
    S.red = reinterpret_cast<double*>(p); p += sizeof(double) * 2 * NW * 4;
    S.redm = reinterpret_cast<double*>(p); p += sizeof(double) * NW * 4;
    p = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(p) + 15) & ~uintptr_t(15));
    GJSmem G = carve_gj<NT>(p, Nmax);

    for (int i = tid; i < 2 * Ns; i += NT) S.fock[i] = J.fock[size_t(w) * 2 * Ns + i];
    for (int i = tid; i < 2 * Nmax; i += NT) S.part[i] = J.part[size_t(w) * 2 * Nmax + i];
    for (int i = tid; i < 4 * Ns; i += NT) S.nbr[i] = J.nbr[i];
    {
        const cx<T>* cg = Tab<T>::coef(J) + size_t(w) * 4 * Ns;   // [fl][sub][orbital]
        for (int i = tid; i < 4 * Nmax; i += NT) {
            const int fl = i / (2 * Nmax), sub = (i / Nmax) & 1, f = i % Nmax;
            S.coef[i] = cg[(size_t(fl) * 2 + sub) * Ns + 2 * f];
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
    const double inv_ns = 1.0 / double(Ns);

    for (uint64_t s = 0; s < nsteps; ++s, k += 4) {
        uint32_t x[4], y[4];
        philox_call(J.seed, wid, 0, k >> 1, x);
        philox_call(J.seed, wid, 0, (k >> 1) + 1, y);
        const double u1 = u01(x[0], x[1]), u2 = u01(x[2], x[3]), u4 = u01(y[2], y[3]);
        const int v1 = int(double(Ns) * u1);
        const int v2 = S.nbr[v1 * 4 + int(4.0 * u2)];
        const int f1 = S.fock[v1] >= 0 ? 0 : 1;
        const int f2 = S.fock[v2] >= 0 ? 0 : 1;
        int kind = 0, accepted;
        double ratio = 1.0;
        if (f1 == f2) {
            accepted = 1;   // ratio m_weight/m_state_weight = 1 (MetroMC.cpp:41 with u4 < 1)
            ++c_noop;
        } else {
            kind = 1;
            const int upf = (f1 == 0) ? v1 : v2, upt = (f1 == 0) ? v2 : v1;
            const int dnf = upt, dnt = upf;
            const int cu = S.fock[upf], cd = S.fock[Ns + dnf];
            cx<T> au = {T(0), T(0)}, ad = {T(0), T(0)};
            for (int f = tid; f < N0; f += NT) {
                const cx<T> u = phi_at<T>(phase, S.coef, J.Nk, Nmax, L, upt, f);
                const cx<T> a = A0[size_t(cu) * N0 + f];
                S.uu[f] = u;
                S.row[f] = a;
                cmac(au, a, u);
            }
            for (int f = tid; f < N1; f += NT) {
                const cx<T> u = phi_at<T>(phase, S.coef + 2 * Nmax, J.Nk, Nmax, L, dnt, f);
                const cx<T> a = A1[size_t(cd) * N1 + f];
                S.uu[Nmax + f] = u;
                S.row[Nmax + f] = a;
                cmac(ad, a, u);
            }
            au = warp_sum(au);
            ad = warp_sum(ad);
            double* rb = S.red + rbuf * NW * 4;
            rbuf ^= 1;
            if (lane == 0) { rb[warp * 4 + 0] = au.x; rb[warp * 4 + 1] = au.y; rb[warp * 4 + 2] = ad.x; rb[warp * 4 + 3] = ad.y; }
            __syncthreads();
            cx<T> ru = {T(0), T(0)}, rd = {T(0), T(0)};
            for (int q = 0; q < NW; ++q) {
                ru.x += T(rb[q * 4 + 0]); ru.y += T(rb[q * 4 + 1]);
                rd.x += T(rb[q * 4 + 2]); rd.y += T(rb[q * 4 + 3]);
            }
            const cx<double> q = to_d(ru) * to_d(rd);
            ratio = norm2(q);
            if (!isfinite(ratio)) { status = GV_ERR_NAN; break; }
            accepted = ratio > 1.0 ? (u4 < 1.0) : (u4 < ratio);
            if (!accepted) {
                ++c_rej;
            } else {
                if (norm2(to_d(ru)) < 1e-9 || norm2(to_d(rd)) < 1e-9) { status = GV_ERR_SINGULAR; break; }
                // w = Ai u - e_c (warp per row)
                for (int pr = warp; pr < N0; pr += NW) {
                    cx<T> a = {T(0), T(0)};
                    const cx<T>* r = A0 + size_t(pr) * N0;
                    for (int f = lane; f < N0; f += 32) cmac(a, r[f], S.uu[f]);
                    a = warp_sum(a);
                    if (lane == 0) { if (pr == cu) a.x -= T(1); S.wv[pr] = a; }
                }
                for (int pr = warp; pr < N1; pr += NW) {
                    cx<T> a = {T(0), T(0)};
                    const cx<T>* r = A1 + size_t(pr) * N1;
                    for (int f = lane; f < N1; f += 32) cmac(a, r[f], S.uu[Nmax + f]);
                    a = warp_sum(a);
                    if (lane == 0) { if (pr == cd) a.x -= T(1); S.wv[Nmax + pr] = a; }
                }
                __syncthreads();
                const cx<T> iu = cinv(ru), id = cinv(rd);
                for (int f = tid; f < N0; f += NT) {
                    const cx<T> rr = S.row[f] * iu;
                    const cx<T> nr = {-rr.x, -rr.y};
                    for (int pr = 0; pr < N0; ++pr) {
                        cx<T> a = A0[size_t(pr) * N0 + f];
                        cmac(a, S.wv[pr], nr);
                        A0[size_t(pr) * N0 + f] = a;
                    }
                }
                for (int f = tid; f < N1; f += NT) {
                    const cx<T> rr = S.row[Nmax + f] * id;
                    const cx<T> nr = {-rr.x, -rr.y};
                    for (int pr = 0; pr < N1; ++pr) {
                        cx<T> a = A1[size_t(pr) * N1 + f];
                        cmac(a, S.wv[Nmax + pr], nr);
                        A1[size_t(pr) * N1 + f] = a;
                    }
                }
                __syncthreads();
                if (tid == 0) {
                    S.fock[upt] = int16_t(cu); S.fock[upf] = -1; S.part[cu] = int16_t(upt);
                    S.fock[Ns + dnt] = int16_t(cd); S.fock[Ns + dnf] = -1; S.part[Nmax + cd] = int16_t(dnt);
                }
                am = am * q;
                amp_normalise(am, ae);
                ++c_acc;
                ++since;
                __syncthreads();
                if (J.reinv_every > 0 && since >= J.reinv_every) {
                    cx<double>* M = J.scratch64 + size_t(w) * Nmax * Nmax;
                    int st = reinvert_walker<T, NT>(J, w, M, G, S.part);
                    if (st != GV_OK) { status = st; break; }
                    am = J.amp_m[w];   // written by thread 0; visible after the block barrier in reinvert
                    __syncthreads();
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
            t.ratio = ratio; t.u4 = u4;
            J.trace[s] = t;
        }
        const uint64_t gs = s0 + s;
        if (meas && (meas == 1 || gs % meas == 0) && mask) {
            // ProjHeis (ProjHeis.cpp:40-158): E/site sample
            if (mask & GV_MEAS_PROJHEIS) {
                cx<double> e = {0.0, 0.0};
                for (int ed = warp; ed < 2 * Ns; ed += NW) {
                    const int vi = J.edges[2 * ed], vj = J.edges[2 * ed + 1];
                    const bool ui = S.fock[vi] >= 0, uj = S.fock[vj] >= 0;
                    if (ui == uj) { if (lane == 0) e.x += 0.25; continue; }
                    const int upf = ui ? vi : vj, upt = ui ? vj : vi;
                    const cx<T> ru = warp_ratio<T>(J, A0, phase, S.coef, N0, S.fock[upf], upt);
                    const cx<T> rd = warp_ratio<T>(J, A1, phase, S.coef + 2 * Nmax, N1, S.fock[Ns + upt], upf);
                    if (lane == 0) {
                        const cx<double> r = to_d(ru) * to_d(rd);
                        e.x += -0.25 - 0.5 * r.x;
                        e.y += -0.5 * r.y;
                    }
                }
                if (lane == 0) { S.redm[warp * 4] = e.x; S.redm[warp * 4 + 1] = e.y; }
                __syncthreads();
                if (tid == 0) {
                    cx<double> t = {0.0, 0.0};
                    for (int q = 0; q < NW; ++q) { t.x += S.redm[q * 4]; t.y += S.redm[q * 4 + 1]; }
                    cx<double>& acc = J.pj[size_t(w) * 2];
                    acc.x += t.x * inv_ns;
                    acc.y += t.y * inv_ns;
                    J.pj[size_t(w) * 2 + 1].x += 1.0;
                    J.pj_n[w] += 1;
                }
                __syncthreads();
            }
            // StagMagnZ (StagMagnZ.cpp:12-43)
            if (mask & GV_MEAS_STAGMAGN) {
                int m = 0;
                for (int v = tid; v < Ns; v += NT) {
                    const int sg = (((v % L) + (v / L)) & 1) ? -1 : 1;
                    m += sg * (S.fock[v] >= 0 ? 1 : -1);
                }
#pragma unroll
                for (int o = 16; o; o >>= 1) m += __shfl_xor_sync(0xffffffffu, m, o);
                if (lane == 0) S.redm[warp * 4 + 2] = double(m);
                __syncthreads();
                if (tid == 0) {
                    double t = 0;
                    for (int q = 0; q < NW; ++q) t += S.redm[q * 4 + 2];
                    J.sm[w].x += t * inv_ns;
                    J.sm_n[w] += 1;
                }
                __syncthreads();
            }
        }
    }
    __syncthreads();
    for (int i = tid; i < 2 * Ns; i += NT) J.fock[size_t(w) * 2 * Ns + i] = S.fock[i];
    for (int i = tid; i < 2 * Nmax; i += NT) J.part[size_t(w) * 2 * Nmax + i] = S.part[i];
    if (tid == 0) {
        J.rng_next[w] = k;
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

// ------------------------------------------------------------------------
// StatSpinStruct (StatSpinStruct.cpp:16-135), ground state: for every pair
// i <= j of the walker's configuration, szz +-1/4 and, for antiparallel
// pairs, s-+ / s+- -= r_up(p_i -> j) r_dn(q_j -> i) (the swap ratio; the
// conj(amp) swamp / w factor of the reference is that ratio).
template <typename T, int NT>
__global__ void __launch_bounds__(NT) k_statspin(DevJob J)
{
    const int w = blockIdx.x;
    if (w >= J.W || J.status[w] != GV_OK) return;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    constexpr int NW = NT / 32;
    const int Ns = J.Ns, Nmax = J.Nmax;
    const int16_t* fock = J.fock + size_t(w) * 2 * Ns;
    const cx<T>* phase = Tab<T>::phase(J);
    const cx<T>* cg = Tab<T>::coef(J) + size_t(w) * 4 * Ns;
    extern __shared__ __align__(16) char smem[];
    cx<T>* coef = reinterpret_cast<cx<T>*>(smem);   // 2 fl * 2 sub * Nmax
    for (int i = tid; i < 4 * Nmax; i += NT) {
        const int fl = i / (2 * Nmax), sub = (i / Nmax) & 1, f = i % Nmax;
        coef[i] = cg[(size_t(fl) * 2 + sub) * Ns + 2 * f];
    }
    __syncthreads();
    const cx<T>* A0 = ai_ptr<T>(J, 0, w);
    const cx<T>* A1 = ai_ptr<T>(J, 1, w);
    double* szz = J.ss;
    double* spm = J.ss + 2 * size_t(Ns) * Ns;
    double* smp = J.ss + 4 * size_t(Ns) * Ns;
    for (int idx = warp; idx < Ns * Ns; idx += NW) {
        const int vi = idx / Ns, vj = idx % Ns;
        if (vj < vi) continue;
        const bool ui = fock[vi] >= 0, uj = fock[vj] >= 0;
        const size_t ij = size_t(vi) * Ns + vj, ji = size_t(vj) * Ns + vi;
        if (ui == uj) {
            if (lane == 0) {
                if (vi == vj) {
                    atomicAdd(&szz[2 * ij], 0.25);
                    atomicAdd(ui ? &spm[2 * ij] : &smp[2 * ij], 1.0);
                } else {
                    atomicAdd(&szz[2 * ij], 0.25);
                    atomicAdd(&szz[2 * ji], 0.25);
                }
            }
            continue;
        }
        const int upf = ui ? vi : vj, upt = ui ? vj : vi;
        const cx<T> ru = warp_ratio<T>(J, A0, phase, coef, J.N[0], fock[upf], upt);
        const cx<T> rd = warp_ratio<T>(J, A1, phase, coef + 2 * Nmax, J.N[1], fock[Ns + upt], upf);
        if (lane == 0) {
            const cx<double> r = to_d(ru) * to_d(rd);
            atomicAdd(&szz[2 * ij], -0.25);
            atomicAdd(&szz[2 * ji], -0.25);
            double* a = ui ? smp : spm;   // vi up: s-+[ij], s+-[ji]; vi down: s+-[ij], s-+[ji]
            double* b = ui ? spm : smp;
            atomicAdd(&a[2 * ij], -r.x); atomicAdd(&a[2 * ij + 1], -r.y);
            atomicAdd(&b[2 * ji], -r.x); atomicAdd(&b[2 * ji + 1], -r.y);
        }
    }
    if (tid == 0) atomicAdd(J.ss_n, 1);
    (void)lane;
}

// ------------------------------------------------------------------------
// VirtUpdate-style ratios for explicit hop sets of one walker (ground state).
template <typename T>
__global__ void k_virt_update(DevJob J, int w, int nset, const int32_t* hops, double* out)
{
    const int lane = threadIdx.x & 31;
    const int set = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
    if (set >= nset) return;
    const int Ns = J.Ns, Nmax = J.Nmax;
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
        const cx<T>* row = ai_ptr<T>(J, fl, w) + size_t(c) * N;
        cx<T> acc = {T(0), T(0)};
        const int sub = sublattice(to, J.L);
        for (int f = lane; f < N; f += 32)
            cmac(acc, row[f], cmul_rn(phase[size_t(to) * J.Nk + f], cg[(size_t(fl) * 2 + sub) * Ns + 2 * f]));
        acc = warp_sum(acc);
        r = r * to_d(acc);
        (void)Nmax;
    }
    if (lane == 0) { out[2 * set] = r.x; out[2 * set + 1] = r.y; }
}

// max |(A Ai)_{f f'} - delta| per walker/flavour in FP64.
template <typename T, int NT>
__global__ void __launch_bounds__(NT) k_drift(DevJob J, double* out)
{
    const int w = blockIdx.x, fl = blockIdx.y;
    const int N = J.N[fl], Ns = J.Ns;
    const int16_t* part = J.part + (size_t(w) * 2 + fl) * J.Nmax;
    const cx<double>* coef = J.coef64 + (size_t(w) * 2 + fl) * 2 * Ns;
    const cx<T>* Ai = ai_ptr<T>(J, fl, w);
    double mx = 0.0;
    for (int idx = threadIdx.x; idx < N * N; idx += NT) {
        const int f = idx / N, g = idx % N;
        cx<double> s = {0.0, 0.0};
        for (int pr = 0; pr < N; ++pr) {
            const int site = part[pr];
            const cx<double> a = cmul_rn(J.phase64[size_t(site) * J.Nk + f], coef[size_t(sublattice(site, J.L)) * Ns + 2 * f]);
            cmac(s, a, to_d(Ai[size_t(pr) * N + g]));
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

// ==========================================================================
// Host side

struct gv_job {
    gv_job_config cfg{};
    Lattice lat;
    Orbitals orb;
    Channel ch;
    int Ns = 0, Nk = 0, Nmax = 0, W = 0;
    int N[2] = {0, 0};
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    DevJob d{};
    std::vector<void*> allocs;
    bool ready = false;
    int nt = 128;
    double last_ms = 0.0;
    int64_t last_launches = 0;
    int64_t total_launches = 0;
    int64_t timer_launch0 = 0;
    cudaEvent_t tev0 = nullptr, tev1 = nullptr;
    std::vector<double> wphi, wneel;
    std::vector<uint64_t> start_draws;   // Philox stream-1 uniform index per walker
};

namespace {

#define GV_CK(x)                                                   \
    do {                                                           \
        cudaError_t e_ = (x);                                      \
        if (e_ != cudaSuccess) {                                   \
            return e_ == cudaErrorMemoryAllocation ? GV_ERR_OOM : GV_ERR_CUDA; \
        }                                                          \
    } while (0)

template <typename P>
gv_status dalloc(gv_job* j, P** ptr, size_t bytes)
{
    void* p = nullptr;
    GV_CK(cudaMalloc(&p, bytes ? bytes : 16));
    GV_CK(cudaMemsetAsync(p, 0, bytes ? bytes : 16, j->stream));
    j->allocs.push_back(p);
    *ptr = static_cast<P*>(p);
    return GV_OK;
}

bool valid_config(const gv_job_config* c)
{
    if (!c) return false;
    if (c->L < 4 || c->L > 64 || (c->L % 2)) return false;
    if (c->channel != GV_CH_GROUNDSTATE) return false;
    if (c->n_walkers < 1 || c->n_walkers > (1 << 20)) return false;
    if (c->precision != GV_PREC_FP64 && c->precision != GV_PREC_MIXED) return false;
    if (c->reinv_every < 0) return false;
    return true;
}

int pick_threads(int Nmax) { return Nmax > 128 ? 256 : 128; }

size_t scratch_walkers(const gv_job* j) { return size_t(j->W); }

template <typename T, int NT>
gv_status launch_walk(gv_job* j, uint64_t nsteps, uint64_t s0, uint64_t meas, int mask)
{
    size_t sm = walk_smem_bytes<T, NT>(j->Ns, j->Nmax);
    GV_CK(cudaFuncSetAttribute(k_walk_gs<T, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm)));
    k_walk_gs<T, NT><<<j->W, NT, sm, j->stream>>>(j->d, nsteps, s0, meas, mask);
    GV_CK(cudaGetLastError());
    ++j->last_launches;
    ++j->total_launches;
    return GV_OK;
}

gv_status walk_dispatch(gv_job* j, uint64_t nsteps, uint64_t s0, uint64_t meas, int mask)
{
    const bool fp64 = j->cfg.precision == GV_PREC_FP64;
    if (j->nt == 128) return fp64 ? launch_walk<double, 128>(j, nsteps, s0, meas, mask)
                                  : launch_walk<float, 128>(j, nsteps, s0, meas, mask);
    return fp64 ? launch_walk<double, 256>(j, nsteps, s0, meas, mask)
                : launch_walk<float, 256>(j, nsteps, s0, meas, mask);
}

gv_status statspin_dispatch(gv_job* j)
{
    const bool fp64 = j->cfg.precision == GV_PREC_FP64;
    size_t sm = (fp64 ? sizeof(cx<double>) : sizeof(cx<float>)) * 4 * j->Nmax;
    if (fp64) k_statspin<double, 128><<<j->W, 128, sm, j->stream>>>(j->d);
    else k_statspin<float, 128><<<j->W, 128, sm, j->stream>>>(j->d);
    GV_CK(cudaGetLastError());
    ++j->last_launches;
    ++j->total_launches;
    return GV_OK;
}

template <typename T, int NT>
gv_status launch_invert(gv_job* j)
{
    size_t sm = gj_smem_bytes(j->Nmax, NT) + 64;
    GV_CK(cudaFuncSetAttribute(k_invert<T, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm)));
    k_invert<T, NT><<<j->W, NT, sm, j->stream>>>(j->d, 0, j->W);
    GV_CK(cudaGetLastError());
    ++j->total_launches;
    return GV_OK;
}

gv_status invert_all(gv_job* j)
{
    return j->cfg.precision == GV_PREC_FP64 ? launch_invert<double, 256>(j) : launch_invert<float, 256>(j);
}

// LatticeState::RanInit (LatticeState.cpp:37-82) for the two-flavour
// half-filled lattice: flavour-0 sites drawn uniformly (Philox stream 1)
// until N0 distinct, the rest flavour 1.
void ran_init(gv_job* j, int w, int8_t* up)
{
    const uint32_t wid = j->cfg.walker_base + uint32_t(w);
    std::fill(up, up + j->Ns, int8_t(0));
    int np = 0;
    uint64_t& k = j->start_draws[w];
    while (np != j->N[0]) {
        int v = int(uniform_at(j->cfg.seed, wid, 1, k++) * double(j->Ns));
        if (!up[v]) { up[v] = 1; ++np; }
    }
}

gv_status upload_configs(gv_job* j, const std::vector<int8_t>& up)
{
    const int Ns = j->Ns, Nmax = j->Nmax;
    std::vector<int16_t> fock(size_t(j->W) * 2 * Ns, -1), part(size_t(j->W) * 2 * Nmax, -1);
    for (int w = 0; w < j->W; ++w) {
        int pc[2] = {0, 0};
        for (int v = 0; v < Ns; ++v) {
            const int fl = up[size_t(w) * Ns + v] ? 0 : 1;   // State::InitFock: particles by ascending site
            fock[(size_t(w) * 2 + fl) * Ns + v] = int16_t(pc[fl]);
            part[(size_t(w) * 2 + fl) * Nmax + pc[fl]] = int16_t(v);
            ++pc[fl];
        }
        if (pc[0] != j->N[0] || pc[1] != j->N[1]) return GV_ERR_INVALID;
    }
    GV_CK(cudaMemcpyAsync(j->d.fock, fock.data(), fock.size() * sizeof(int16_t), cudaMemcpyHostToDevice, j->stream));
    GV_CK(cudaMemcpyAsync(j->d.part, part.data(), part.size() * sizeof(int16_t), cudaMemcpyHostToDevice, j->stream));
    return GV_OK;
}

}  // namespace

extern "C" {

const char* gv_version(void) { return "gpvmc_gb300 0.1 (sm_103a)"; }

gv_status gv_phi_table(int32_t L, double phi, double neel, double neel_exp, const double* bc, int32_t fl, double* out)
{
    if (L < 2 || L > 64 || (L % 2) || !bc || fl < 0 || fl > 1 || !out) return GV_ERR_INVALID;
    Orbitals o = make_orbitals(L, bc[0], bc[1]);
    if (!o.ok) return GV_ERR_INVALID;
    std::vector<zd> ph, coef(size_t(2) * o.Ns);
    phase_table(o, ph);
    if (!stagflux_coefs(o, phi, neel, neel_exp, fl, coef.data())) return GV_ERR_NAN;
    for (int orb = 0; orb < o.Ns; ++orb)
        for (int s = 0; s < o.Ns; ++s) {
            const int sub = ((s % L) + (s / L)) & 1;
            zd v = phi_elem(ph[size_t(s) * o.Nk + orb / 2], coef[size_t(sub) * o.Ns + orb]);
            out[2 * (size_t(orb) * o.Ns + s)] = v.real();
            out[2 * (size_t(orb) * o.Ns + s) + 1] = v.imag();
        }
    return GV_OK;
}

gv_status gv_lattice_neighbours(int32_t L, int32_t* nbr)
{
    if (L < 2 || L > 64 || !nbr) return GV_ERR_INVALID;
    Lattice lat = make_square_lattice(L);
    std::memcpy(nbr, lat.nbr.data(), sizeof(int32_t) * lat.nbr.size());
    return GV_OK;
}

gv_status gv_channel_orbitals(int32_t L, const double* bc, int32_t channel, const int32_t* q, int32_t fl,
                              int32_t* orb, int32_t* N, int32_t* Nexc)
{
    if (L < 2 || L > 64 || (L % 2) || !bc || !q || fl < 0 || fl > 1) return GV_ERR_INVALID;
    if (channel != GV_CH_GROUNDSTATE && channel != GV_CH_TRANS) return GV_ERR_INVALID;
    Orbitals o = make_orbitals(L, bc[0], bc[1]);
    if (!o.ok) return GV_ERR_INVALID;
    Channel ch = make_channel(o, channel, q[0], q[1]);
    if (!ch.ok) return GV_ERR_INVALID;
    if (N) *N = ch.N[fl];
    if (Nexc) *Nexc = ch.Nexc;
    if (orb)
        for (int x = 0; x < o.Ns; ++x)
            if (ch.fock0[fl][x] < ch.N[fl]) orb[ch.fock0[fl][x]] = x;
    return GV_OK;
}

void gv_philox4x32_10(const uint32_t* c, const uint32_t* k, uint32_t* out)
{
    philox4x32_10(c[0], c[1], c[2], c[3], k[0], k[1], out);
}

double gv_uniform_at(uint64_t seed, uint32_t walker, uint32_t stream, uint64_t k)
{
    return uniform_at(seed, walker, stream, k);
}

const char* gv_status_string(gv_status s)
{
    switch (s) {
        case GV_OK: return "ok";
        case GV_ERR_INVALID: return "invalid argument or unsupported configuration";
        case GV_ERR_SINGULAR: return "singular Slater matrix";
        case GV_ERR_NAN: return "NaN or Inf encountered";
        case GV_ERR_ZERO_AMP: return "zero overlap";
        case GV_ERR_DRIFT: return "inverse drift above threshold";
        case GV_ERR_TIMEOUT: return "device wait timed out";
        case GV_ERR_OOM: return "device allocation failed";
        case GV_ERR_CUDA: return "CUDA runtime error";
        case GV_ERR_NOT_READY: return "walkers not initialised";
        default: return "unknown status";
    }
}

gv_status gv_job_footprint(const gv_job_config* c, uint64_t* bytes)
{
    if (!valid_config(c) || !bytes) return GV_ERR_INVALID;
    const uint64_t Ns = uint64_t(c->L) * c->L, Nk = Ns / 2, W = c->n_walkers;
    const uint64_t N0 = Ns / 2, N1 = Ns / 2, Nmax = std::max(N0, N1);
    const uint64_t es = c->precision == GV_PREC_FP64 ? 16 : 8;
    uint64_t b = 0;
    b += Ns * Nk * (16 + 8);                 // phase tables
    b += W * 4 * Ns * (16 + 8);              // coefficients
    b += W * (N0 * N0 + N1 * N1) * es;       // inverses
    b += W * (2 * Ns + 2 * Nmax) * 2;        // occupancy
    b += W * 256;                            // per-walker scalars
    b += W * Nmax * Nmax * 16;               // FP64 re-inversion scratch
    b += 5 * Ns * Ns * 16;                   // StatSpinStruct sums
    *bytes = b;
    return GV_OK;
}

gv_status gv_job_create(const gv_job_config* cfg, gv_job** out)
{
    if (!out) return GV_ERR_INVALID;
    *out = nullptr;
    if (!valid_config(cfg)) return GV_ERR_INVALID;
    gv_job* j = new gv_job;
    j->cfg = *cfg;
    const int L = cfg->L;
    j->lat = make_square_lattice(L);
    j->orb = make_orbitals(L, cfg->phase_shift[0], cfg->phase_shift[1]);
    if (!j->orb.ok) { delete j; return GV_ERR_INVALID; }
    j->ch = make_channel(j->orb, 0, cfg->q[0], cfg->q[1]);
    if (!j->ch.ok) { delete j; return GV_ERR_INVALID; }
    j->Ns = L * L;
    j->Nk = j->orb.Nk;
    j->N[0] = j->ch.N[0];
    j->N[1] = j->ch.N[1];
    j->Nmax = std::max(j->N[0], j->N[1]);
    j->W = cfg->n_walkers;
    j->nt = pick_threads(j->Nmax);
    j->start_draws.assign(j->W, 0);

    // Per-walker variational parameters (Philox stream 2, uniforms 0 and 1).
    j->wphi.assign(j->W, cfg->phi);
    j->wneel.assign(j->W, cfg->neel);
    for (int w = 0; w < j->W; ++w) {
        const uint32_t wid = cfg->walker_base + uint32_t(w);
        if (cfg->phi_range[1] > cfg->phi_range[0])
            j->wphi[w] = cfg->phi_range[0] + (cfg->phi_range[1] - cfg->phi_range[0]) * uniform_at(cfg->seed, wid, 2, 0);
        if (cfg->neel_range[1] > cfg->neel_range[0])
            j->wneel[w] = cfg->neel_range[0] + (cfg->neel_range[1] - cfg->neel_range[0]) * uniform_at(cfg->seed, wid, 2, 1);
    }
    // Host tables.
    std::vector<zd> ph;
    phase_table(j->orb, ph);
    std::vector<zd> coef(size_t(j->W) * 4 * j->Ns);
    for (int w = 0; w < j->W; ++w)
        for (int fl = 0; fl < 2; ++fl)
            if (!stagflux_coefs(j->orb, j->wphi[w], j->wneel[w], cfg->neel_exp, fl, &coef[(size_t(w) * 2 + fl) * 2 * j->Ns])) {
                delete j;
                return GV_ERR_NAN;
            }
    std::vector<cx<double>> ph64(ph.size());
    std::vector<cx<float>> ph32(ph.size());
    for (size_t i = 0; i < ph.size(); ++i) {
        ph64[i] = {ph[i].real(), ph[i].imag()};
        ph32[i] = {float(ph[i].real()), float(ph[i].imag())};
    }
    std::vector<cx<double>> cf64(coef.size());
    std::vector<cx<float>> cf32(coef.size());
    for (size_t i = 0; i < coef.size(); ++i) {
        cf64[i] = {coef[i].real(), coef[i].imag()};
        cf32[i] = {float(coef[i].real()), float(coef[i].imag())};
    }
    std::vector<int32_t> edges(size_t(2) * j->Ns * 2);
    for (int e = 0; e < 2 * j->Ns; ++e) { edges[2 * e] = j->lat.edge_i[e]; edges[2 * e + 1] = j->lat.edge_j[e]; }

    auto fail = [&](gv_status s) { gv_job_destroy(j); return s; };
    if (cudaStreamCreateWithFlags(&j->stream, cudaStreamNonBlocking) != cudaSuccess) { delete j; return GV_ERR_CUDA; }
    if (cudaEventCreate(&j->ev0) != cudaSuccess || cudaEventCreate(&j->ev1) != cudaSuccess) return fail(GV_ERR_CUDA);

    DevJob& d = j->d;
    d.L = L; d.Ns = j->Ns; d.Nk = j->Nk; d.Nexc = 1; d.W = j->W;
    d.N[0] = j->N[0]; d.N[1] = j->N[1]; d.Nmax = j->Nmax;
    d.precision = cfg->precision; d.channel = cfg->channel;
    d.seed = cfg->seed; d.walker_base = cfg->walker_base; d.reinv_every = cfg->reinv_every;
    d.trace = nullptr; d.trace_walker = -1;
    const size_t es = cfg->precision == GV_PREC_FP64 ? sizeof(cx<double>) : sizeof(cx<float>);
    gv_status st = GV_OK;
    int32_t *nbr = nullptr, *edg = nullptr;
    cx<double>* p64 = nullptr; cx<float>* p32 = nullptr; cx<double>* c64 = nullptr; cx<float>* c32 = nullptr;
    void *a0 = nullptr, *a1 = nullptr;
    if ((st = dalloc(j, &nbr, sizeof(int32_t) * 4 * j->Ns)) ||
        (st = dalloc(j, &edg, edges.size() * sizeof(int32_t))) ||
        (st = dalloc(j, &p64, ph64.size() * sizeof(cx<double>))) ||
        (st = dalloc(j, &p32, ph32.size() * sizeof(cx<float>))) ||
        (st = dalloc(j, &c64, cf64.size() * sizeof(cx<double>))) ||
        (st = dalloc(j, &c32, cf32.size() * sizeof(cx<float>))) ||
        (st = dalloc(j, &a0, size_t(j->W) * j->N[0] * j->N[0] * es)) ||
        (st = dalloc(j, &a1, size_t(j->W) * j->N[1] * j->N[1] * es)) ||
        (st = dalloc(j, &d.fock, size_t(j->W) * 2 * j->Ns * sizeof(int16_t))) ||
        (st = dalloc(j, &d.part, size_t(j->W) * 2 * j->Nmax * sizeof(int16_t))) ||
        (st = dalloc(j, &d.amp_m, size_t(j->W) * sizeof(cx<double>))) ||
        (st = dalloc(j, &d.amp_e, size_t(j->W) * sizeof(int32_t))) ||
        (st = dalloc(j, &d.rng_next, size_t(j->W) * sizeof(uint64_t))) ||
        (st = dalloc(j, &d.counts, size_t(j->W) * 5 * sizeof(unsigned long long))) ||
        (st = dalloc(j, &d.since_reinv, size_t(j->W) * sizeof(int32_t))) ||
        (st = dalloc(j, &d.status, size_t(j->W) * sizeof(int32_t))) ||
        (st = dalloc(j, &d.pj, size_t(j->W) * 2 * sizeof(cx<double>))) ||
        (st = dalloc(j, &d.pj_n, size_t(j->W) * sizeof(int32_t))) ||
        (st = dalloc(j, &d.sm, size_t(j->W) * sizeof(cx<double>))) ||
        (st = dalloc(j, &d.sm_n, size_t(j->W) * sizeof(int32_t))) ||
        (st = dalloc(j, &d.ss, size_t(5) * j->Ns * j->Ns * 2 * sizeof(double))) ||
        (st = dalloc(j, &d.ss_n, sizeof(int32_t))) ||
        (st = dalloc(j, &d.scratch64, scratch_walkers(j) * j->Nmax * j->Nmax * sizeof(cx<double>))))
        return fail(st);
    d.nbr = nbr; d.edges = edg; d.phase64 = p64; d.phase32 = p32; d.coef64 = c64; d.coef32 = c32;
    d.Ai[0] = a0; d.Ai[1] = a1;
    if (cudaMemcpyAsync(nbr, j->lat.nbr.data(), sizeof(int32_t) * 4 * j->Ns, cudaMemcpyHostToDevice, j->stream) ||
        cudaMemcpyAsync(edg, edges.data(), edges.size() * sizeof(int32_t), cudaMemcpyHostToDevice, j->stream) ||
        cudaMemcpyAsync(p64, ph64.data(), ph64.size() * sizeof(cx<double>), cudaMemcpyHostToDevice, j->stream) ||
        cudaMemcpyAsync(p32, ph32.data(), ph32.size() * sizeof(cx<float>), cudaMemcpyHostToDevice, j->stream) ||
        cudaMemcpyAsync(c64, cf64.data(), cf64.size() * sizeof(cx<double>), cudaMemcpyHostToDevice, j->stream) ||
        cudaMemcpyAsync(c32, cf32.data(), cf32.size() * sizeof(cx<float>), cudaMemcpyHostToDevice, j->stream) ||
        cudaStreamSynchronize(j->stream))
        return fail(GV_ERR_CUDA);
    *out = j;
    return GV_OK;
}

gv_status gv_job_destroy(gv_job* j)
{
    if (!j) return GV_OK;
    if (j->stream) cudaStreamSynchronize(j->stream);
    for (void* p : j->allocs) cudaFree(p);
    if (j->ev0) cudaEventDestroy(j->ev0);
    if (j->tev0) cudaEventDestroy(j->tev0);
    if (j->tev1) cudaEventDestroy(j->tev1);
    if (j->ev1) cudaEventDestroy(j->ev1);
    if (j->stream) cudaStreamDestroy(j->stream);
    delete j;
    return GV_OK;
}

gv_status gv_job_dims(const gv_job* j, int32_t* Ns, int32_t* Nup, int32_t* Ndn, int32_t* Nexc)
{
    if (!j) return GV_ERR_INVALID;
    if (Ns) *Ns = j->Ns;
    if (Nup) *Nup = j->N[0];
    if (Ndn) *Ndn = j->N[1];
    if (Nexc) *Nexc = 1;
    return GV_OK;
}

gv_status gv_job_set_meas_mask(gv_job* j, int32_t mask)
{
    if (!j || (mask & ~(GV_MEAS_PROJHEIS | GV_MEAS_STAGMAGN | GV_MEAS_STATSPIN))) return GV_ERR_INVALID;
    j->cfg.meas_mask = mask;
    return GV_OK;
}

gv_status gv_job_init_walkers(gv_job* j, const int8_t* up)
{
    if (!j) return GV_ERR_INVALID;
    const int Ns = j->Ns, W = j->W;
    std::vector<int8_t> cfg(size_t(W) * Ns);
    std::vector<int> pending;
    if (up) {
        std::memcpy(cfg.data(), up, cfg.size());
        for (int w = 0; w < W; ++w) {
            int c = 0;
            for (int v = 0; v < Ns; ++v) c += cfg[size_t(w) * Ns + v] ? 1 : 0;
            if (c != j->N[0]) return GV_ERR_INVALID;
        }
    } else {
        std::fill(j->start_draws.begin(), j->start_draws.end(), 0);
        for (int w = 0; w < W; ++w) ran_init(j, w, &cfg[size_t(w) * Ns]);
    }
    std::vector<int32_t> status(W, GV_OK);
    GV_CK(cudaMemsetAsync(j->d.status, 0, sizeof(int32_t) * W, j->stream));
    GV_CK(cudaMemsetAsync(j->d.rng_next, 0, sizeof(uint64_t) * W, j->stream));
    GV_CK(cudaMemsetAsync(j->d.counts, 0, sizeof(unsigned long long) * 5 * W, j->stream));
    GV_CK(cudaMemsetAsync(j->d.since_reinv, 0, sizeof(int32_t) * W, j->stream));
    // vmc.cpp:221-241: up to 10 random starts until the amplitude is non-zero.
    for (int attempt = 0; attempt < 10; ++attempt) {
        gv_status st = upload_configs(j, cfg);
        if (st) return st;
        st = invert_all(j);
        if (st) return st;
        GV_CK(cudaMemcpyAsync(status.data(), j->d.status, sizeof(int32_t) * W, cudaMemcpyDeviceToHost, j->stream));
        GV_CK(cudaStreamSynchronize(j->stream));
        bool again = false;
        for (int w = 0; w < W; ++w)
            if (status[w] == GV_ERR_SINGULAR && !up) { ran_init(j, w, &cfg[size_t(w) * Ns]); again = true; }
        if (!again) break;
        if (attempt == 9) return GV_ERR_SINGULAR;
        GV_CK(cudaMemsetAsync(j->d.status, 0, sizeof(int32_t) * W, j->stream));
    }
    for (int w = 0; w < W; ++w)
        if (status[w] != GV_OK) { j->ready = true; return status[w]; }
    j->ready = true;
    return GV_OK;
}

static gv_status walk_impl(gv_job* j, uint64_t len, uint64_t meas, gv_trace* dtrace, int trace_walker)
{
    if (!j) return GV_ERR_INVALID;
    if (!j->ready) return GV_ERR_NOT_READY;
    const int mask = meas ? j->cfg.meas_mask : 0;
    j->d.trace = dtrace;
    j->d.trace_walker = trace_walker;
    j->last_launches = 0;
    if (meas) {
        GV_CK(cudaMemsetAsync(j->d.pj, 0, sizeof(cx<double>) * 2 * j->W, j->stream));
        GV_CK(cudaMemsetAsync(j->d.pj_n, 0, sizeof(int32_t) * j->W, j->stream));
        GV_CK(cudaMemsetAsync(j->d.sm, 0, sizeof(cx<double>) * j->W, j->stream));
        GV_CK(cudaMemsetAsync(j->d.sm_n, 0, sizeof(int32_t) * j->W, j->stream));
        GV_CK(cudaMemsetAsync(j->d.ss, 0, sizeof(double) * 10 * j->Ns * j->Ns, j->stream));
        GV_CK(cudaMemsetAsync(j->d.ss_n, 0, sizeof(int32_t), j->stream));
    }
    GV_CK(cudaEventRecord(j->ev0, j->stream));
    gv_status st = GV_OK;
    if (!(mask & GV_MEAS_STATSPIN)) {
        st = walk_dispatch(j, len, 0, meas, mask);
    } else {
        // Split at the measurement points: steps [a, b) then measure after b-1.
        uint64_t a = 0;
        while (a < len && !st) {
            uint64_t m = (a == 0) ? 0 : ((a + meas - 1) / meas) * meas;   // next s with s % meas == 0, s >= a
            if (j->d.trace) j->d.trace = dtrace + a;
            if (m >= len) { st = walk_dispatch(j, len - a, a, 0, 0); a = len; break; }
            // run steps a..m (inclusive) with in-kernel ProjHeis/StagMagnZ at m
            const uint64_t nsteps = m - a + 1;
            st = walk_dispatch(j, nsteps, a, meas, mask & ~GV_MEAS_STATSPIN);
            if (!st) st = statspin_dispatch(j);
            a = m + 1;
        }
        j->d.trace = dtrace;
    }
    GV_CK(cudaEventRecord(j->ev1, j->stream));
    j->d.trace = nullptr;
    j->d.trace_walker = -1;
    return st;
}

gv_status gv_job_walk(gv_job* j, uint64_t len, uint64_t meas) { return walk_impl(j, len, meas, nullptr, -1); }

gv_status gv_job_walk_traced(gv_job* j, uint64_t len, uint64_t meas, int32_t walker, gv_trace* trace)
{
    if (!j || !trace || walker < 0 || walker >= j->W) return GV_ERR_INVALID;
    gv_trace* dt = nullptr;
    GV_CK(cudaMalloc(&dt, sizeof(gv_trace) * (len ? len : 1)));
    gv_status st = walk_impl(j, len, meas, dt, walker);
    if (!st) {
        if (cudaMemcpyAsync(trace, dt, sizeof(gv_trace) * len, cudaMemcpyDeviceToHost, j->stream) ||
            cudaStreamSynchronize(j->stream))
            st = GV_ERR_CUDA;
    }
    cudaFree(dt);
    return st ? st : gv_job_synchronize(j);
}

gv_status gv_job_synchronize(gv_job* j)
{
    if (!j) return GV_ERR_INVALID;
    GV_CK(cudaStreamSynchronize(j->stream));
    float ms = 0;
    if (cudaEventElapsedTime(&ms, j->ev0, j->ev1) == cudaSuccess) j->last_ms = ms;
    std::vector<int32_t> status(j->W);
    GV_CK(cudaMemcpy(status.data(), j->d.status, sizeof(int32_t) * j->W, cudaMemcpyDeviceToHost));
    for (int32_t s : status)
        if (s) return s;
    return GV_OK;
}

gv_status gv_job_timer_start(gv_job* j)
{
    if (!j) return GV_ERR_INVALID;
    if (!j->tev0) {
        GV_CK(cudaEventCreate(&j->tev0));
        GV_CK(cudaEventCreate(&j->tev1));
    }
    j->timer_launch0 = j->total_launches;
    GV_CK(cudaEventRecord(j->tev0, j->stream));
    return GV_OK;
}

gv_status gv_job_timer_stop(gv_job* j, double* ms, int64_t* launches)
{
    if (!j || !j->tev0) return GV_ERR_INVALID;
    GV_CK(cudaEventRecord(j->tev1, j->stream));
    GV_CK(cudaEventSynchronize(j->tev1));
    float f = 0;
    GV_CK(cudaEventElapsedTime(&f, j->tev0, j->tev1));
    if (ms) *ms = f;
    if (launches) *launches = j->total_launches - j->timer_launch0;
    return GV_OK;
}

gv_status gv_job_last_walk_ms(gv_job* j, double* ms, int64_t* launches)
{
    if (!j) return GV_ERR_INVALID;
    if (ms) *ms = j->last_ms;
    if (launches) *launches = j->last_launches;
    return GV_OK;
}

gv_status gv_job_reinvert(gv_job* j)
{
    if (!j) return GV_ERR_INVALID;
    if (!j->ready) return GV_ERR_NOT_READY;
    gv_status st = invert_all(j);
    if (st) return st;
    GV_CK(cudaMemsetAsync(j->d.since_reinv, 0, sizeof(int32_t) * j->W, j->stream));
    return gv_job_synchronize(j);
}

gv_status gv_job_drift(gv_job* j, double* out)
{
    if (!j || !out) return GV_ERR_INVALID;
    if (!j->ready) return GV_ERR_NOT_READY;
    double* d = nullptr;
    GV_CK(cudaMalloc(&d, sizeof(double) * 2 * j->W));
    if (j->cfg.precision == GV_PREC_FP64) k_drift<double, 256><<<dim3(j->W, 2), 256, 0, j->stream>>>(j->d, d);
    else k_drift<float, 256><<<dim3(j->W, 2), 256, 0, j->stream>>>(j->d, d);
    cudaError_t e = cudaGetLastError();
    if (!e) e = cudaMemcpyAsync(out, d, sizeof(double) * 2 * j->W, cudaMemcpyDeviceToHost, j->stream);
    if (!e) e = cudaStreamSynchronize(j->stream);
    cudaFree(d);
    return e ? GV_ERR_CUDA : GV_OK;
}

gv_status gv_job_virt_update(gv_job* j, int32_t walker, int32_t nset, const int32_t* hops, double* out)
{
    if (!j || !hops || !out || walker < 0 || walker >= j->W || nset < 0) return GV_ERR_INVALID;
    if (!j->ready) return GV_ERR_NOT_READY;
    if (nset == 0) return GV_OK;
    for (int i = 0; i < 4 * nset; ++i)
        if (hops[i] < -1 || hops[i] >= j->Ns) return GV_ERR_INVALID;
    int32_t* dh = nullptr;
    double* dout = nullptr;
    GV_CK(cudaMalloc(&dh, sizeof(int32_t) * 4 * nset));
    if (cudaMalloc(&dout, sizeof(double) * 2 * nset)) { cudaFree(dh); return GV_ERR_OOM; }
    cudaError_t e = cudaMemcpyAsync(dh, hops, sizeof(int32_t) * 4 * nset, cudaMemcpyHostToDevice, j->stream);
    const int per = 4;
    if (!e) {
        if (j->cfg.precision == GV_PREC_FP64)
            k_virt_update<double><<<(nset + per - 1) / per, 32 * per, 0, j->stream>>>(j->d, walker, nset, dh, dout);
        else
            k_virt_update<float><<<(nset + per - 1) / per, 32 * per, 0, j->stream>>>(j->d, walker, nset, dh, dout);
        e = cudaGetLastError();
    }
    if (!e) e = cudaMemcpyAsync(out, dout, sizeof(double) * 2 * nset, cudaMemcpyDeviceToHost, j->stream);
    if (!e) e = cudaStreamSynchronize(j->stream);
    cudaFree(dh);
    cudaFree(dout);
    return e ? GV_ERR_CUDA : GV_OK;
}

gv_status gv_job_read_config(gv_job* j, int8_t* up)
{
    if (!j || !up) return GV_ERR_INVALID;
    GV_CK(cudaStreamSynchronize(j->stream));
    std::vector<int16_t> fock(size_t(j->W) * 2 * j->Ns);
    GV_CK(cudaMemcpy(fock.data(), j->d.fock, fock.size() * sizeof(int16_t), cudaMemcpyDeviceToHost));
    for (int w = 0; w < j->W; ++w)
        for (int v = 0; v < j->Ns; ++v) up[size_t(w) * j->Ns + v] = fock[size_t(w) * 2 * j->Ns + v] >= 0 ? 1 : 0;
    return GV_OK;
}

gv_status gv_job_read_particles(gv_job* j, int32_t walker, int32_t fl, int32_t* out)
{
    if (!j || !out || walker < 0 || walker >= j->W || fl < 0 || fl > 1) return GV_ERR_INVALID;
    GV_CK(cudaStreamSynchronize(j->stream));
    std::vector<int16_t> part(j->Nmax);
    GV_CK(cudaMemcpy(part.data(), j->d.part + (size_t(walker) * 2 + fl) * j->Nmax, sizeof(int16_t) * j->Nmax,
                     cudaMemcpyDeviceToHost));
    for (int p = 0; p < j->N[fl]; ++p) out[p] = part[p];
    return GV_OK;
}

gv_status gv_job_read_amplitude(gv_job* j, double* mant, int32_t* exp10)
{
    if (!j || !mant || !exp10) return GV_ERR_INVALID;
    GV_CK(cudaStreamSynchronize(j->stream));
    std::vector<cx<double>> m(j->W);
    std::vector<int32_t> e(j->W);
    GV_CK(cudaMemcpy(m.data(), j->d.amp_m, sizeof(cx<double>) * j->W, cudaMemcpyDeviceToHost));
    GV_CK(cudaMemcpy(e.data(), j->d.amp_e, sizeof(int32_t) * j->W, cudaMemcpyDeviceToHost));
    for (int w = 0; w < j->W; ++w) {
        const double a = std::hypot(m[w].x, m[w].y);
        if (a == 0.0) { mant[2 * w] = mant[2 * w + 1] = 0.0; exp10[w] = 0; continue; }
        const double l10 = std::log10(a) + e[w] * std::log10(2.0);
        double fe = std::floor(l10);
        const double scale = std::pow(10.0, l10 - fe) / a;
        double re = m[w].x * scale, im = m[w].y * scale;
        if (std::hypot(re, im) >= 10.0) { re /= 10.0; im /= 10.0; fe += 1; }
        mant[2 * w] = re;
        mant[2 * w + 1] = im;
        exp10[w] = int32_t(fe);
    }
    return GV_OK;
}

gv_status gv_job_read_inverse(gv_job* j, int32_t walker, int32_t fl, double* out)
{
    if (!j || !out || walker < 0 || walker >= j->W || fl < 0 || fl > 1) return GV_ERR_INVALID;
    GV_CK(cudaStreamSynchronize(j->stream));
    const int N = j->N[fl];
    const size_t n = size_t(N) * N;
    if (j->cfg.precision == GV_PREC_FP64) {
        std::vector<cx<double>> a(n);
        GV_CK(cudaMemcpy(a.data(), static_cast<cx<double>*>(j->d.Ai[fl]) + size_t(walker) * n, n * sizeof(cx<double>),
                         cudaMemcpyDeviceToHost));
        for (int p = 0; p < N; ++p)
            for (int f = 0; f < N; ++f) {
                out[2 * (size_t(p) + size_t(f) * N)] = a[size_t(p) * N + f].x;
                out[2 * (size_t(p) + size_t(f) * N) + 1] = a[size_t(p) * N + f].y;
            }
    } else {
        std::vector<cx<float>> a(n);
        GV_CK(cudaMemcpy(a.data(), static_cast<cx<float>*>(j->d.Ai[fl]) + size_t(walker) * n, n * sizeof(cx<float>),
                         cudaMemcpyDeviceToHost));
        for (int p = 0; p < N; ++p)
            for (int f = 0; f < N; ++f) {
                out[2 * (size_t(p) + size_t(f) * N)] = a[size_t(p) * N + f].x;
                out[2 * (size_t(p) + size_t(f) * N) + 1] = a[size_t(p) * N + f].y;
            }
    }
    return GV_OK;
}

gv_status gv_job_read_counts(gv_job* j, uint64_t* counts)
{
    if (!j || !counts) return GV_ERR_INVALID;
    GV_CK(cudaStreamSynchronize(j->stream));
    GV_CK(cudaMemcpy(counts, j->d.counts, sizeof(uint64_t) * 5 * j->W, cudaMemcpyDeviceToHost));
    return GV_OK;
}

gv_status gv_job_read_state_index(gv_job* j, int32_t* state)
{
    if (!j || !state) return GV_ERR_INVALID;
    for (int w = 0; w < j->W; ++w) state[w] = 0;
    return GV_OK;
}

gv_status gv_job_read_projheis(gv_job* j, double* vals, int32_t* nmeas)
{
    if (!j || !vals) return GV_ERR_INVALID;
    GV_CK(cudaStreamSynchronize(j->stream));
    GV_CK(cudaMemcpy(vals, j->d.pj, sizeof(cx<double>) * 2 * j->W, cudaMemcpyDeviceToHost));
    if (nmeas) GV_CK(cudaMemcpy(nmeas, j->d.pj_n, sizeof(int32_t) * j->W, cudaMemcpyDeviceToHost));
    return GV_OK;
}

gv_status gv_job_read_stagmagn(gv_job* j, double* vals, int32_t* nmeas)
{
    if (!j || !vals) return GV_ERR_INVALID;
    GV_CK(cudaStreamSynchronize(j->stream));
    GV_CK(cudaMemcpy(vals, j->d.sm, sizeof(cx<double>) * j->W, cudaMemcpyDeviceToHost));
    if (nmeas) GV_CK(cudaMemcpy(nmeas, j->d.sm_n, sizeof(int32_t) * j->W, cudaMemcpyDeviceToHost));
    return GV_OK;
}

gv_status gv_job_read_statspin(gv_job* j, double* vals, int32_t* nmeas)
{
    if (!j || !vals) return GV_ERR_INVALID;
    GV_CK(cudaStreamSynchronize(j->stream));
    GV_CK(cudaMemcpy(vals, j->d.ss, sizeof(double) * 10 * j->Ns * j->Ns, cudaMemcpyDeviceToHost));
    if (nmeas) GV_CK(cudaMemcpy(nmeas, j->d.ss_n, sizeof(int32_t), cudaMemcpyDeviceToHost));
    return GV_OK;
}

}  // extern "C"
