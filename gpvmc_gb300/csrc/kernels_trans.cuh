// Engine kernels for the transverse-exciton channel (StagFluxTransExciton,
// StagFluxTransExciton.cpp:7-44).  Included by engine.cu after kernels.cuh.
//
// Channel state k of momentum q fills the lower band for both flavours, adds
// the upper-band orbital exc_up[k] to flavour 0 (N0 = Ns/2 + 1 particles) and
// removes the lower-band orbital exc_dn[k] from flavour 1 (N1 = Ns/2 - 1).
// From the current state `cur`, state k != cur is one orbital hop per flavour:
//     flavour 0: exc_up[cur] -> exc_up[k]   (Slater row r0 = wslot0[exc_up[cur]], same for all k)
//     flavour 1: exc_dn[k] -> exc_dn[cur]   (row r_k = wslot1[exc_dn[k]], same new orbital for all k)
// so LatticeStepper::trystep's VirtUpdate over all Nexc states (LatticeStepper.cpp:36-100;
// SlaterDeterminant.cpp:96-268) is a column replacement (the moved particle)
// plus one row replacement per flavour, whose determinant ratio by the
// 2x2 determinant lemma of linalg::DetUpdate (linalg.cpp:107-400) is
//     rho_k = M11 (R_k A^-1 e_r) - (A^-1)(c, r) (R_k A^-1 C - R_k[c])
// with M11 = (A^-1 C)_c the column-only ratio.  With the per-walker overlap
// rows kept current,
//     GupT[f][k] = sum_p phi_{exc_up[k]}(x_p) (A0^-1)(p, f)    (Nexc x N0)
//     g[f]       = sum_p phi_{exc_dn[cur]}(x_p) (A1^-1)(p, f)  (N1)
// a proposal moving the flavour-0 particle c0 to t0 and the flavour-1
// particle c1 to t1 costs one Nexc x N0 product Z_k = sum_f GupT[f][k] phi_f(t0):
//     rho0_k = M11_0 GupT[r0][k] - (A0^-1)(c0, r0) (Z_k - phi_{exc_up[k]}(t0))
//     rho1_k = M11_1 g[r_k] - (A1^-1)(c1, r_k) (sum_f g[f] phi_f(t1) - phi_{exc_dn[cur]}(t1))
// and the Metropolis ratio is sum_k |rho0_k rho1_k|^2 / sigma, sigma being the
// accepted state's weight over |det_0 det_1|^2.  An accepted move applies
// linalg::InvUpdate's rank-2 (column + row) Woodbury update (linalg.cpp:402-573)
// to both inverses and the same rank-2 change to GupT and g, so no O(N^3)
// work happens between re-inversions.
#pragma once

#include "kernels.cuh"

namespace gv {
namespace {


// Number of occupied orbitals strictly between a and b in one flavour's
// wavefunction Fock state (slot table wslot_fl), by one warp.
__device__ __forceinline__ int warp_count_between(const int16_t* wslot_fl, int a, int b)
{
    const int lane = threadIdx.x & 31;
    const int lo = (a < b ? a : b) + 1, hi = a > b ? a : b;
    int n = 0;
    for (int x = lo + lane; x < hi; x += 32) n += wslot_fl[x] >= 0 ? 1 : 0;
#pragma unroll
    for (int o = 16; o; o >>= 1) n += __shfl_xor_sync(0xffffffffu, n, o);
    return n;
}

// Overlap of every channel state with the current one, relative to the
// current amplitude: rho0_k = GupT[r0][k] g[r_k] (k != cur), 1 (k = cur).
// out[w*Nexc + k] = |rho0_k|^2 (when out is given) and sigma[w] = sum_k.
// Used to pick the start state of largest |Amp| (vmc.cpp:243-263) and for
// the stepper's weight (LatticeStepper::weight, LatticeStepper.cpp:149-169).
template <typename T, int NT>
__global__ void __launch_bounds__(NT) k_trans_overlaps(DevJob J, double* out)
{
    constexpr int NW = NT / 32;
    const int w = blockIdx.x;
    if (w >= J.W || J.status[w] != GV_OK) return;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int Ns = J.Ns, Nexc = J.Nexc, N0 = J.N[0];
    const int cur = J.cur[w];
    const int16_t* wslot = J.wslot + size_t(w) * 2 * Ns;
    const cx<T>* G = static_cast<const cx<T>*>(J.gup) + size_t(w) * N0 * Nexc;
    const cx<T>* g = static_cast<const cx<T>*>(J.gdn) + size_t(w) * J.Nmax;
    const int r0 = max(int(wslot[J.exc_up[cur]]), 0);
    double s = 0.0;
    for (int k = tid; k < Nexc; k += NT) {
        double n = 1.0;
        if (k != cur) n = norm2(to_d(G[size_t(r0) * Nexc + k]) * to_d(g[wslot[Ns + J.exc_dn[k]]]));
        if (out) out[size_t(w) * Nexc + k] = n;
        s += n;
    }
    __shared__ double red[NW];
#pragma unroll
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) red[warp] = s;
    __syncthreads();
    if (tid == 0) {
        double t = 0.0;
        for (int q = 0; q < NW; ++q) t += red[q];
        J.sigma[w] = t;
    }
}

// max |(A^-1)_ij| over both flavours, per walker.
template <typename T, int NT>
__global__ void __launch_bounds__(NT) k_inverse_max_abs(DevJob J, double* out)
{
    const int w = blockIdx.x;
    if (w >= J.W) return;
    double m = 0.0;
    for (int fl = 0; fl < 2; ++fl) {
        const cx<T>* A = ai_ptr<T>(J, fl, w);
        const int n = J.N[fl] * J.N[fl];
        for (int i = threadIdx.x; i < n; i += NT) m = fmax(m, double(fmax(fabs(A[i].x), fabs(A[i].y))));
    }
    __shared__ double red[NT / 32];
#pragma unroll
    for (int o = 16; o; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int q = 0; q < NT / 32; ++q) t = fmax(t, red[q]);
        out[w] = t;
    }
}

struct TransLayout {
    size_t fock, part, wslot, worb, nbr, exu, exd, coef, C, rowc, g, Y, zp, phk, ru, rd, zc, dk, ak, bk, X, Yv,
        red, gj, total;
};

template <typename T, int NT>
__host__ __device__ inline TransLayout trans_layout(int Ns, int Nmax, int Nexc, bool gj)
{
    TransLayout l;
    size_t b = 0;
    auto al = [&](size_t x) { b = (b + 15) & ~size_t(15); size_t r = b; b += x; return r; };
    const size_t c = sizeof(cx<T>);
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
    l.zp = al(c * 2 * Nexc);
    l.phk = al(c * Nexc);
    l.ru = al(c * Nexc);
    l.rd = al(c * Nexc);
    l.zc = al(c * Nmax);
    l.dk = al(c * Nexc);
    l.ak = al(c * Nexc);
    l.bk = al(c * Nexc);
    l.X = al(c * 2 * Nmax);
    l.Yv = al(c * 2 * Nmax);
    l.red = al(sizeof(double) * 2 * 8 * (NT / 32) + sizeof(int) * (NT / 32));
    l.gj = al(gj ? gj_smem_bytes(Nmax, NT) : 16);
    l.total = al(16);
    return l;
}

// 2x2 complex inverse (row-major m[0..3]) with its determinant.
template <typename T>
__device__ __forceinline__ cx<T> inv2(const cx<T> m[4], cx<T> mi[4])
{
    const cx<T> det = m[0] * m[3] - m[1] * m[2];
    const cx<T> id = cinv(det);
    mi[0] = m[3] * id;
    mi[1] = cneg(m[1]) * id;
    mi[2] = cneg(m[2]) * id;
    mi[3] = m[0] * id;
    return det;
}

// Column p of AiT: AiT[f][p] -= wa * X[f] + wb * Y[f] (rank-2), 8 loads in flight.
template <typename T>
__device__ __forceinline__ void col_update2(cx<T>* A, int N, int p, cx<T> wa, const cx<T>* X, cx<T> wb,
                                            const cx<T>* Y, bool two)
{
    const cx<T> na = cneg(wa), nb = cneg(wb);
    int f = 0;
    for (; f + 8 <= N; f += 8) {
        cx<T> a[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) a[k] = A[size_t(f + k) * N + p];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            cmac(a[k], na, X[f + k]);
            if (two) cmac(a[k], nb, Y[f + k]);
            A[size_t(f + k) * N + p] = a[k];
        }
    }
    for (; f < N; ++f) {
        cx<T> a = A[size_t(f) * N + p];
        cmac(a, na, X[f]);
        if (two) cmac(a, nb, Y[f]);
        A[size_t(f) * N + p] = a;
    }
}

// ------------------------------------------------------------------------
// Metropolis walk, exciton channel: one CTA per walker, MetroMC::Step
// (MetroMC.cpp:90-103) with LatticeStepper::trystep / step
// (LatticeStepper.cpp:36-147).  Uniform order and no-op handling as the
// ground-state kernel; the proposal's weight is the sum over channel states
// and the accepted move hops the wavefunction to the arg-max state
// (first maximum, as trystep's scan), applying State::Hop's sign
// (State.cpp:73-115) to the amplitude.
template <typename T, int NT>
__global__ void __launch_bounds__(NT, 2) k_walk_trans(DevJob J, uint64_t nsteps, int inkernel_reinv)
{
    extern __shared__ __align__(16) char smem[];
    constexpr int NW = NT / 32;
    const int w = blockIdx.x;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (w >= J.W || J.status[w] != GV_OK) return;
    const bool forced = J.forced_walker >= 0;
    if (forced && w != J.forced_walker) return;
    const int Ns = J.Ns, Nmax = J.Nmax, L = J.L, Nk = J.Nk, Nexc = J.Nexc;
    const int N0 = J.N[0], N1 = J.N[1];
    const TransLayout lay = trans_layout<T, NT>(Ns, Nmax, Nexc, inkernel_reinv != 0);
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
    cx<T>* s_zc = reinterpret_cast<cx<T>*>(smem + lay.zc);
    cx<T>* s_dk = reinterpret_cast<cx<T>*>(smem + lay.dk);
    cx<T>* s_ak = reinterpret_cast<cx<T>*>(smem + lay.ak);
    cx<T>* s_bk = reinterpret_cast<cx<T>*>(smem + lay.bk);
    cx<T>* s_X = reinterpret_cast<cx<T>*>(smem + lay.X);
    cx<T>* s_Yv = reinterpret_cast<cx<T>*>(smem + lay.Yv);
    double* s_red = reinterpret_cast<double*>(smem + lay.red);

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
        const cx<T>* cg = Tab<T>::coef(J) + size_t(w) * 4 * Ns;   // [fl][sub][orbital]
        for (int i = tid; i < 4 * Ns; i += NT) s_coef[i] = cg[i];
    }
    const cx<T>* gglob = static_cast<const cx<T>*>(J.gdn) + size_t(w) * Nmax;
    for (int i = tid; i < N1; i += NT) s_g[i] = gglob[i];
    __syncthreads();

    const cx<T>* phase = Tab<T>::phase(J);
    const cx<T>* cf0 = s_coef;
    const cx<T>* cf1 = s_coef + 2 * Ns;
    cx<T>* A0 = ai_ptr<T>(J, 0, w);
    cx<T>* A1 = ai_ptr<T>(J, 1, w);
    cx<T>* G = static_cast<cx<T>*>(J.gup) + size_t(w) * N0 * Nexc;
    const uint32_t wid = J.walker_base + uint32_t(w);
    uint64_t kk = J.rng_next[w];
    unsigned long long c_acc = 0, c_noop = 0, c_rej = 0, c_reinv = 0;
    int since = J.since_reinv[w];
    cx<double> am = J.amp_m[w];
    int ae = J.amp_e[w];
    int cur = J.cur[w];
    int wsign = J.wsign[w];
    double sigma = J.sigma[w];
    int status = GV_OK;
    int rbuf = 0;
    const int fh = (N0 + 1) >> 1;

    for (uint64_t s = 0; s < nsteps; ++s, kk += 4) {
        uint32_t x[4], y[4];
        philox_call(J.seed, wid, 0, kk >> 1, x);
        philox_call(J.seed, wid, 0, (kk >> 1) + 1, y);
        const uint64_t m4 = u52(y[2], y[3]);
        int v1 = scaled_floor(uint32_t(Ns), u52(x[0], x[1]));
        int v2 = s_nbr[v1 * 4 + int(u52(x[2], x[3]) >> 50)];
        if (forced) { v1 = J.forced_v1; v2 = J.forced_v2; }
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
            // Phase 1: rows c of both inverses, new columns C (phi_{row orbital}(t)),
            // M11 = row_c . C, g . C1, and row r0 of GupT.
            cx<T> m11u = {T(0), T(0)}, m11d = {T(0), T(0)}, gc = {T(0), T(0)};
            for (int f = tid; f < N0; f += NT) {
                const cx<T> a = A0[size_t(f) * N0 + cu];
                const cx<T> c = phi_orb<T>(phase, cf0, Nk, Ns, L, upt, s_worb[f]);
                s_rowc[f] = a;
                s_C[f] = c;
                cmac(m11u, a, c);
            }
            for (int f = tid; f < N1; f += NT) {
                const cx<T> a = A1[size_t(f) * N1 + cd];
                const cx<T> c = phi_orb<T>(phase, cf1, Nk, Ns, L, dnt, s_worb[Nmax + f]);
                s_rowc[Nmax + f] = a;
                s_C[Nmax + f] = c;
                cmac(m11d, a, c);
                cmac(gc, s_g[f], c);
            }
            for (int k = tid; k < Nexc; k += NT) s_Y[k] = G[size_t(r0) * Nexc + k];
            m11u = warp_sum(m11u);
            m11d = warp_sum(m11d);
            gc = warp_sum(gc);
            T* rb = reinterpret_cast<T*>(s_red) + rbuf * NW * 8;
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
            // Phase 2: Z_k = sum_f GupT[f][k] C0[f], two halves of f per state.
            for (int idx = tid; idx < 2 * Nexc; idx += NT) {
                const int k = idx % Nexc, h = idx / Nexc;
                const int fa = h ? fh : 0, fb = h ? N0 : fh;
                cx<T> acc = {T(0), T(0)};
                int f = fa;
                for (; f + 8 <= fb; f += 8) {
                    cx<T> a[8];
#pragma unroll
                    for (int q = 0; q < 8; ++q) a[q] = G[size_t(f + q) * Nexc + k];
#pragma unroll
                    for (int q = 0; q < 8; ++q) cmac(acc, a[q], s_C[f + q]);
                }
                for (; f < fb; ++f) cmac(acc, G[size_t(f) * Nexc + k], s_C[f]);
                s_zp[idx] = acc;
            }
            __syncthreads();
            // Phase 3: per-state ratios, their sum and the first arg-max.
            const cx<T> M12 = s_rowc[r0];
            const cx<T> gcd = gC - phi_orb<T>(phase, cf1, Nk, Ns, L, dnt, hcur);
            T wsum = T(0), wbest = T(-1);
            int kbest = Nexc;
            for (int k = tid; k < Nexc; k += NT) {
                const cx<T> Z = s_zp[k] + s_zp[Nexc + k];
                const cx<T> phk = phi_orb<T>(phase, cf0, Nk, Ns, L, upt, s_exu[k]);
                cx<T> ru = M11u, rd = M11d;
                if (k != cur) {
                    ru = M11u * s_Y[k] - M12 * (Z - phk);
                    const int rk = max(int(s_wslot[Ns + s_exd[k]]), 0);   // occupied for every k != cur
                    rd = M11d * s_g[rk] - s_rowc[Nmax + rk] * gcd;
                }
                s_phk[k] = phk;
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
            khop = (forced && J.forced_khop >= 0 && J.forced_khop < Nexc) ? J.forced_khop : kbest;
            ratio = wsum / T(sigma);
            if (!isfinite(ratio) || khop >= Nexc) { status = GV_ERR_NAN; break; }
            accepted = forced ? J.forced_accept : (ratio > T(1) ? 1 : (Accept<T>::uniform(m4) < ratio));
            if (!accepted) {
                ++c_rej;
            } else {
                const cx<T> rho_u = s_ru[khop], rho_d = s_rd[khop];
                if (norm2(rho_u) < T(1e-9) || norm2(rho_d) < T(1e-9)) { status = GV_ERR_SINGULAR; break; }
                const bool row = khop != cur;
                const int rp = row ? max(int(s_wslot[Ns + s_exd[khop]]), 0) : 0;   // flavour-1 row replaced
                // Stage 1: per-state coefficients of the GupT update and GupT's column khop.
                for (int k = tid; k < Nexc; k += NT) {
                    const cx<T> Z = s_zp[k] + s_zp[Nexc + k];
                    const cx<T> dk = s_phk[k] - phi_orb<T>(phase, cf0, Nk, Ns, L, upf, s_exu[k]);
                    s_dk[k] = dk;
                    s_ak[k] = Z + dk * M11u - s_phk[k];
                    s_bk[k] = s_Y[k] + dk * M12;
                }
                if (row)
                    for (int f = tid; f < N0; f += NT) s_zc[f] = G[size_t(f) * Nexc + khop];
                __syncthreads();
                // Stage 2: capacitance matrices (linalg.cpp:402-573) and the row
                // vectors [X; Y] = M^-1 [row_c; V1] of both flavours.
                cx<T> Mu[4], Mui[4], Md[4], Mdi[4];
                cx<T> delu = {T(0), T(0)}, deld = {T(0), T(0)}, Dh;
                {
                    const cx<T> phc_t = phi_orb<T>(phase, cf1, Nk, Ns, L, dnt, hcur);
                    Dh = phc_t - phi_orb<T>(phase, cf1, Nk, Ns, L, dnf, hcur);
                    if (row) {
                        // flavour 0: R = phi_{exc_up[khop]}(x'), row r0
                        delu = s_C[r0] - phi_orb<T>(phase, cf0, Nk, Ns, L, upf, ocur);
                        const cx<T> Zk = s_zp[khop] + s_zp[Nexc + khop];
                        const cx<T> dkh = s_dk[khop];
                        const cx<T> raic = Zk + dkh * M11u, raier = s_Y[khop] + dkh * M12;
                        Mu[0] = M11u; Mu[1] = M12;
                        Mu[2] = raic - s_phk[khop] - delu * M11u;
                        Mu[3] = raier - delu * M12;
                        inv2(Mu, Mui);
                        // flavour 1: R = phi_{hcur}(x'), row rp holding exc_dn[khop]
                        const cx<T> M12d = s_rowc[Nmax + rp];
                        deld = s_C[Nmax + rp] - phi_orb<T>(phase, cf1, Nk, Ns, L, dnf, s_exd[khop]);
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
                // Stage 3: rank-2 updates.  Column p (one owner thread): its entry
                // in row r before the update, then (A^-1 C)_p - [p == c].
                for (int p = tid; p < N0; p += NT) {
                    const cx<T> h = row ? A0[size_t(r0) * N0 + p] : cx<T>{T(0), T(0)};
                    cx<T> wa = col_dot<T>(A0, N0, p, s_C);
                    if (p == cu) wa.x -= T(1);
                    col_update2<T>(A0, N0, p, wa, s_X, h, s_Yv, row);
                }
                for (int p = tid; p < N1; p += NT) {
                    const cx<T> h = row ? A1[size_t(rp) * N1 + p] : cx<T>{T(0), T(0)};
                    cx<T> wa = col_dot<T>(A1, N1, p, s_C + Nmax);
                    if (p == cd) wa.x -= T(1);
                    col_update2<T>(A1, N1, p, wa, s_X + Nmax, h, s_Yv + Nmax, row);
                }
                // GupT[f][k] += d_k row_c[f] - a_k X[f] - b_k Y[f]
                for (int idx = tid; idx < N0 * Nexc; idx += NT) {
                    const int f = idx / Nexc, k = idx - f * Nexc;
                    cx<T> v = G[idx];
                    cmac(v, s_dk[k], s_rowc[f]);
                    cmac(v, cneg(s_ak[k]), s_X[f]);
                    if (row) cmac(v, cneg(s_bk[k]), s_Yv[f]);
                    G[idx] = v;
                }
                // g of the state after the move (its hole orbital).
                {
                    const cx<T> ah = gC + Dh * M11d - phi_orb<T>(phase, cf1, Nk, Ns, L, dnt, hcur);
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
                    am = am * (to_d(rho_u) * to_d(rho_d));
                    amp_normalise(am, ae);
                }
                if (row) { cur = khop; wsign *= hs; }
                sigma = double(wsum) / double(Accept<T>::ratio(rho_u, rho_d));
                ++c_acc;
                ++since;
                __syncthreads();
                if (inkernel_reinv && J.reinv_every > 0 && since >= J.reinv_every) {
                    char* gp = smem + lay.gj;
                    GJSmem GS = carve_gj<NT>(gp, Nmax);
                    cx<double>* M = J.scratch64 + size_t(w) * Nmax * Nmax;
                    const int st = reinvert_walker<T, NT>(J, w, M, GS, s_part, s_worb);
                    if (st != GV_OK) { status = st; break; }
                    trans_rebuild<T, NT>(J, w, s_part, cur);
                    for (int i = tid; i < N1; i += NT) s_g[i] = gglob[i];
                    am = J.amp_m[w];
                    ae = J.amp_e[w];
                    since = 0;
                    ++c_reinv;
                    __syncthreads();
                }
            }
        }
        if (J.trace && w == J.trace_walker && tid == 0) {
            gv_trace t;
            t.v1 = v1; t.v2 = v2; t.kind = kind; t.accepted = accepted; t.khop = kind ? khop : -1; t.pad = 0;
            t.ratio = double(ratio); t.u4 = u01(y[2], y[3]);
            J.trace[s] = t;
        }
        if (forced && !J.forced_accept) return;   // evaluation only: nothing was changed, nothing to write
    }
    __syncthreads();
    for (int i = tid; i < 2 * Ns; i += NT) {
        J.fock[size_t(w) * 2 * Ns + i] = s_fock[i];
        J.wslot[size_t(w) * 2 * Ns + i] = s_wslot[i];
    }
    for (int i = tid; i < 2 * Nmax; i += NT) {
        J.part[size_t(w) * 2 * Nmax + i] = s_part[i];
        J.worb[size_t(w) * 2 * Nmax + i] = s_worb[i];
    }
    cx<T>* gout = static_cast<cx<T>*>(J.gdn) + size_t(w) * Nmax;
    for (int i = tid; i < N1; i += NT) gout[i] = s_g[i];
    if (tid == 0) {
        if (!forced) J.rng_next[w] = kk;   // single-walker stepping draws its uniforms itself
        unsigned long long* c = J.counts + size_t(w) * 5;
        c[0] += c_acc + c_noop + c_rej;
        c[1] += c_acc;
        c[2] += c_noop;
        c[3] += c_rej;
        c[4] += c_reinv;
        J.since_reinv[w] = since;
        J.amp_m[w] = am;
        J.amp_e[w] = ae;
        J.cur[w] = cur;
        J.wsign[w] = wsign;
        J.sigma[w] = sigma;
        J.status[w] = status;
    }
}

// ------------------------------------------------------------------------
// ProjHeis in the exciton channel (ProjHeis.cpp:40-158, Nexc > 1) and
// StagMagnZ.  For every antiparallel bond b (flavour-0 particle at u moves to
// the flavour-1 site d and back) and every state k the swap ratio
// rho_k(b) = rho0_k(b) rho1_k(b) follows the proposal formulas above, with
// Z_k(d) = sum_f GupT[f][k] phi_f(d) evaluated in tiles of flavour-1 sites
// (an Nexc x N0 x N1 product per measurement).  With a_k = hs_k rho0_k the
// state overlaps (hs_k the wavefunction hop sign) and
//     h_k = hs_k (rho0_k (n_par - n_anti) / 4 - sum_b rho_k(b) / 2),
// H_{k1 k2} += conj(a_k1) h_k2 / w and O_{k1 k2} += conj(a_k1) a_k2 / w,
// w = sum_k |a_k|^2 (the stepper weight over |Amp|^2).
constexpr int kMeasTile = 8;

struct MeasLayout {
    size_t fock, part, wslot, worb, nbr, exu, exd, coef, rq, h, Y, g, gcs, Ct, arow, bond, S, a, hh, f32, red, total;
};

template <typename T, int NT>
__host__ __device__ inline MeasLayout meas_layout(int Ns, int Nmax, int Nexc)
{
    MeasLayout l;
    size_t b = 0;
    auto al = [&](size_t x) { b = (b + 15) & ~size_t(15); size_t r = b; b += x; return r; };
    const size_t c = sizeof(cx<T>);
    l.fock = al(sizeof(int16_t) * 2 * Ns);
    l.part = al(sizeof(int16_t) * 2 * Nmax);
    l.wslot = al(sizeof(int16_t) * 2 * Ns);
    l.worb = al(sizeof(int16_t) * 2 * Nmax);
    l.nbr = al(sizeof(int16_t) * 4 * Ns);
    l.exu = al(sizeof(int16_t) * Nexc);
    l.exd = al(sizeof(int16_t) * Nexc);
    l.coef = al(c * 4 * Ns);
    l.rq = al(c * 4 * Ns);
    l.h = al(c * Nmax);
    l.Y = al(c * Nexc);
    l.g = al(c * Nmax);
    l.gcs = al(c * Ns);
    l.Ct = al(c * kMeasTile * Nmax);
    l.arow = al(c * kMeasTile * Nexc);
    l.bond = al(c * 4 * kMeasTile * 4);   // per tile bond: M11_0, M12, M11_1, g.C1 - phi_h
    l.S = al(sizeof(cx<double>) * Nexc);
    l.a = al(sizeof(cx<double>) * Nexc);
    l.hh = al(sizeof(cx<double>) * Nexc);
    l.f32 = al(sizeof(cx<float>) * 3 * Nexc);   // FP32 factors of the H / O outer products (mixed form)
    l.red = al(sizeof(double) * 4 * (NT / 32) + 16);
    l.total = al(16);
    return l;
}

// H / O of a mixed job in blocks of measurements.  A measurement leaves its
// FP32 factors caf = conj(a) / w, hf = h, af = a (each Nexc long) in the
// walker's next slot; n waiting slots fold as
//     dst[k1 k2] = src[k1 k2] + fp64( sum_{m < n} caf_m[k1] hf_m[k2] )
// (and O with af): the block sum in FP32 (FMA, m ascending), then one exact
// widening and one FP64 add per entry.  Per entry, component and block the
// FP32 sum is off by at most 2n 2^-24 sum_m |caf_m[k1]| |hf_m[k2]| (two FMA
// roundings per term, each at most 2^-24 of a partial sum): 4e-6 of the
// block's absolute sum for n = 32.  Each thread owns 4 rows k1 of one column
// k2: the column's factors are coalesced loads, the rows' are broadcasts.
template <int NT>
__device__ void ho_fold(const cx<float>* slots, int n, int Nexc, const cx<double>* src, cx<double>* dst)
{
    constexpr int KB = 4;
    const size_t NN = size_t(Nexc) * Nexc;
    const int nkb = (Nexc + KB - 1) / KB;
    for (int t = threadIdx.x; t < nkb * Nexc; t += NT) {
        const int k2 = t % Nexc, k1b = (t / Nexc) * KB;
        cx<float> h[KB], o[KB];
#pragma unroll
        for (int i = 0; i < KB; ++i) h[i] = o[i] = cx<float>{0.f, 0.f};
        for (int m = 0; m < n; ++m) {
            const cx<float>* s = slots + size_t(m) * 3 * Nexc;
            const cx<float> hv = s[Nexc + k2], av = s[2 * Nexc + k2];
#pragma unroll
            for (int i = 0; i < KB; ++i)
                if (k1b + i < Nexc) {
                    const cx<float> ca = s[k1b + i];
                    cmac(h[i], ca, hv);
                    cmac(o[i], ca, av);
                }
        }
#pragma unroll
        for (int i = 0; i < KB; ++i)
            if (k1b + i < Nexc) {
                const size_t idx = size_t(k1b + i) * Nexc + k2;
                const cx<double> a = src[idx], b = src[NN + idx];
                dst[idx] = cx<double>{a.x + f32_to_f64(h[i].x), a.y + f32_to_f64(h[i].y)};
                dst[NN + idx] = cx<double>{b.x + f32_to_f64(o[i].x), b.y + f32_to_f64(o[i].y)};
            }
    }
}

// One measurement's factors (f: 3*Nexc in shared memory) into walker w's next
// slot; the kHoSlots-th folds the block into the walker's FP64 sums.
template <int NT>
__device__ void ho_push(const DevJob& J, int w, const cx<float>* f)
{
    const int Nexc = J.Nexc;
    const int n = J.pxs_n[w];
    cx<float>* slots = J.pxs + size_t(w) * kHoSlots * 3 * Nexc;
    for (int i = threadIdx.x; i < 3 * Nexc; i += NT) slots[size_t(n) * 3 * Nexc + i] = f[i];
    __syncthreads();   // the slot's stores are visible to the whole block
    if (n + 1 == kHoSlots) {
        cx<double>* H = J.pjx + size_t(w) * 2 * Nexc * Nexc;
        ho_fold<NT>(slots, kHoSlots, Nexc, H, H);
    }
    if (threadIdx.x == 0) J.pxs_n[w] = (n + 1) % kHoSlots;
}

// Read-out of the H / O sums of walkers w0 .. w0 + gridDim.x - 1 with their
// waiting slots folded in (into out, one 2*Nexc*Nexc block per walker); the
// job's own sums and slots stay as they are, so what a walk accumulates does
// not depend on when it is read.
template <int NT>
__global__ void __launch_bounds__(NT) k_ho_read(DevJob J, int w0, cx<double>* out)
{
    const int w = w0 + blockIdx.x;
    if (w >= J.W) return;
    const int Nexc = J.Nexc;
    const size_t per = size_t(2) * Nexc * Nexc;
    ho_fold<NT>(J.pxs + size_t(w) * kHoSlots * 3 * Nexc, J.pxs_n[w], Nexc, J.pjx + size_t(w) * per,
                out + size_t(blockIdx.x) * per);
}

template <typename T, int NT>
__global__ void __launch_bounds__(NT) k_measure_trans(DevJob J, int mask, const cx<float>* zpre)
{
    extern __shared__ __align__(16) char smem[];
    constexpr int NW = NT / 32;
    constexpr int TT = kMeasTile;
    const int w = blockIdx.x;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (w >= J.W || J.status[w] != GV_OK) return;
    const int Ns = J.Ns, Nmax = J.Nmax, L = J.L, Nk = J.Nk, Nexc = J.Nexc;
    const int N0 = J.N[0], N1 = J.N[1];
    const MeasLayout lay = meas_layout<T, NT>(Ns, Nmax, Nexc);
    int16_t* s_fock = reinterpret_cast<int16_t*>(smem + lay.fock);
    int16_t* s_part = reinterpret_cast<int16_t*>(smem + lay.part);
    int16_t* s_wslot = reinterpret_cast<int16_t*>(smem + lay.wslot);
    int16_t* s_worb = reinterpret_cast<int16_t*>(smem + lay.worb);
    int16_t* s_nbr = reinterpret_cast<int16_t*>(smem + lay.nbr);
    int16_t* s_exu = reinterpret_cast<int16_t*>(smem + lay.exu);
    int16_t* s_exd = reinterpret_cast<int16_t*>(smem + lay.exd);
    cx<T>* s_coef = reinterpret_cast<cx<T>*>(smem + lay.coef);
    cx<T>* s_rq = reinterpret_cast<cx<T>*>(smem + lay.rq);
    cx<T>* s_h = reinterpret_cast<cx<T>*>(smem + lay.h);
    cx<T>* s_Y = reinterpret_cast<cx<T>*>(smem + lay.Y);
    cx<T>* s_g = reinterpret_cast<cx<T>*>(smem + lay.g);
    cx<T>* s_gcs = reinterpret_cast<cx<T>*>(smem + lay.gcs);
    cx<T>* s_Ct = reinterpret_cast<cx<T>*>(smem + lay.Ct);
    cx<T>* s_arow = reinterpret_cast<cx<T>*>(smem + lay.arow);
    cx<T>* s_bond = reinterpret_cast<cx<T>*>(smem + lay.bond);
    cx<double>* s_S = reinterpret_cast<cx<double>*>(smem + lay.S);
    cx<double>* s_a = reinterpret_cast<cx<double>*>(smem + lay.a);
    cx<double>* s_hh = reinterpret_cast<cx<double>*>(smem + lay.hh);
    double* s_red = reinterpret_cast<double*>(smem + lay.red);

    for (int i = tid; i < 2 * Ns; i += NT) {
        s_fock[i] = J.fock[size_t(w) * 2 * Ns + i];
        s_wslot[i] = J.wslot[size_t(w) * 2 * Ns + i];
    }
    for (int i = tid; i < 2 * Nmax; i += NT) {
        s_part[i] = J.part[size_t(w) * 2 * Nmax + i];
        s_worb[i] = J.worb[size_t(w) * 2 * Nmax + i];
    }
    for (int i = tid; i < 4 * Ns; i += NT) s_nbr[i] = int16_t(J.nbr[i]);
    for (int i = tid; i < Nexc; i += NT) {
        s_exu[i] = J.exc_up[i];
        s_exd[i] = J.exc_dn[i];
        s_S[i] = cx<double>{0.0, 0.0};
    }
    {
        const cx<T>* cg = Tab<T>::coef(J) + size_t(w) * 4 * Ns;
        for (int i = tid; i < 4 * Ns; i += NT) s_coef[i] = cg[i];
    }
    const int cur = J.cur[w];
    __syncthreads();
    const cx<T>* phase = Tab<T>::phase(J);
    const cx<T>* cf0 = s_coef;
    const cx<T>* cf1 = s_coef + 2 * Ns;
    const cx<T>* A0 = ai_ptr<T>(J, 0, w);
    const cx<T>* A1 = ai_ptr<T>(J, 1, w);
    const cx<T>* G = static_cast<const cx<T>*>(J.gup) + size_t(w) * N0 * Nexc;
    const cx<T>* gg = static_cast<const cx<T>*>(J.gdn) + size_t(w) * Nmax;
    const int ocur = s_exu[cur], hcur = s_exd[cur];
    const int r0 = max(int(s_wslot[ocur]), 0);
    const double inv_ns = 1.0 / double(Ns);

    if (mask & GV_MEAS_PROJHEIS) {
        for (int p = tid; p < N0; p += NT) s_h[p] = A0[size_t(r0) * N0 + p];
        for (int k = tid; k < Nexc; k += NT) s_Y[k] = G[size_t(r0) * Nexc + k];
        for (int f = tid; f < N1; f += NT) s_g[f] = gg[f];
        // Pass 1: column-only ratio of every particle to each antiparallel neighbour,
        // rq[site][slot] (as the ground-state ProjHeis).
        for (int idx = tid; idx < N0 + N1; idx += NT) {
            const int fl = idx < N0 ? 0 : 1;
            const int p = fl ? idx - N0 : idx;
            const int N = fl ? N1 : N0;
            const cx<T>* A = fl ? A1 : A0;
            const cx<T>* cf = fl ? cf1 : cf0;
            const int site = s_part[fl * Nmax + p];
            int js[4];
            bool anti[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                js[q] = s_nbr[site * 4 + q];
                anti[q] = (s_fock[js[q]] >= 0) != (fl == 0);
            }
            cx<T> acc[4] = {{T(0), T(0)}, {T(0), T(0)}, {T(0), T(0)}, {T(0), T(0)}};
            for (int f = 0; f < N; ++f) {
                const cx<T> a = A[size_t(f) * N + p];
                const int o = s_worb[fl * Nmax + f];
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    if (anti[q]) cmac(acc[q], a, phi_orb<T>(phase, cf, Nk, Ns, L, js[q], o));
            }
#pragma unroll
            for (int q = 0; q < 4; ++q) s_rq[site * 4 + q] = acc[q];
        }
        __syncthreads();
        // Pass 2: g . C1(u) - phi_h(u) for every flavour-0 site u.
        for (int p = tid; p < N0; p += NT) {
            const int u = s_part[p];
            cx<T> acc = {T(0), T(0)};
            for (int f = 0; f < N1; ++f) cmac(acc, s_g[f], phi_orb<T>(phase, cf1, Nk, Ns, L, u, s_worb[Nmax + f]));
            s_gcs[u] = acc - phi_orb<T>(phase, cf1, Nk, Ns, L, u, hcur);
        }
        __syncthreads();
        // Pass 3: tiles of flavour-1 sites d (targets of the flavour-0 moves).
        // With zpre (the tensor-core product, Z[w][d][k]) the tile's Z values are read.
        for (int t0 = 0; t0 < N1; t0 += TT) {
            const int nt = min(TT, N1 - t0);
            if (!zpre)
                for (int idx = tid; idx < nt * N0; idx += NT) {
                    const int tt = idx / N0, f = idx % N0;
                    s_Ct[tt * Nmax + f] = phi_orb<T>(phase, cf0, Nk, Ns, L, s_part[Nmax + t0 + tt], s_worb[f]);
                }
            for (int idx = tid; idx < nt * Nexc; idx += NT) {
                const int tt = idx / Nexc, k = idx % Nexc;
                const int rk = s_wslot[Ns + s_exd[k]];   // -1 for k = cur (its hole is empty)
                s_arow[tt * Nexc + k] = rk >= 0 ? A1[size_t(rk) * N1 + t0 + tt] : cx<T>{T(0), T(0)};
            }
            for (int idx = tid; idx < nt * 4; idx += NT) {
                const int tt = idx >> 2, q = idx & 3;
                const int d = s_part[Nmax + t0 + tt], u = s_nbr[d * 4 + q];
                cx<T>* B = s_bond + (tt * 4 + q) * 4;
                if (s_fock[u] >= 0) {   // antiparallel bond (u: flavour 0, d: flavour 1)
                    int qu = 0;
                    while (qu < 3 && s_nbr[u * 4 + qu] != d) ++qu;
                    B[0] = s_rq[u * 4 + qu];          // M11_0: flavour-0 particle u -> d
                    B[1] = s_h[s_fock[u]];            // (A0^-1)(c0, r0)
                    B[2] = s_rq[d * 4 + q];           // M11_1: flavour-1 particle d -> u
                    B[3] = s_gcs[u];
                } else {
                    B[0].x = nan("");
                }
            }
            __syncthreads();
            for (int k = tid; k < Nexc; k += NT) {
                cx<T> Z[TT];
#pragma unroll
                for (int tt = 0; tt < TT; ++tt) Z[tt] = {T(0), T(0)};
                if (zpre) {
#pragma unroll
                    for (int tt = 0; tt < TT; ++tt)
                        if (tt < nt) {
                            const cx<float> z = zpre[(size_t(w) * N1 + t0 + tt) * Nexc + k];
                            Z[tt] = cx<T>{T(z.x), T(z.y)};
                        }
                } else {
                    for (int f = 0; f < N0; ++f) {
                        const cx<T> gk = G[size_t(f) * Nexc + k];
#pragma unroll
                        for (int tt = 0; tt < TT; ++tt)
                            if (tt < nt) cmac(Z[tt], gk, s_Ct[tt * Nmax + f]);
                    }
                }
                const int rk = s_wslot[Ns + s_exd[k]];
                cx<double> acc = s_S[k];
                cx<T> part = {T(0), T(0)};   // FP32 form: the tile's bond products, added to acc once
#pragma unroll
                for (int tt = 0; tt < TT; ++tt) {
                    if (tt >= nt) break;
                    const int d = s_part[Nmax + t0 + tt];
                    const cx<T> zc = Z[tt] - phi_orb<T>(phase, cf0, Nk, Ns, L, d, s_exu[k]);
                    for (int q = 0; q < 4; ++q) {
                        const cx<T>* B = s_bond + (tt * 4 + q) * 4;
                        if (isnan(B[0].x)) continue;
                        cx<T> r0k = B[0], r1k = B[2];
                        if (k != cur) {
                            r0k = B[0] * s_Y[k] - B[1] * zc;
                            r1k = B[2] * s_g[rk] - s_arow[tt * Nexc + k] * B[3];
                        }
                        bool wide = true;
                        if constexpr (sizeof(T) == 4) {
                            // FP32 product unless it could come near the FP32 range (then FP64, as the plain form)
                            wide = (fabsf(r0k.x) + fabsf(r0k.y)) * (fabsf(r1k.x) + fabsf(r1k.y)) > 1e30f;
                            if (!wide) cmac(part, r0k, r1k);
                        }
                        if (wide) {
                            const cx<double> r = to_d(r0k) * to_d(r1k);
                            acc.x += r.x;
                            acc.y += r.y;
                        }
                    }
                }
                if constexpr (sizeof(T) == 4) {
                    acc.x += f32_to_f64(part.x);
                    acc.y += f32_to_f64(part.y);
                }
                s_S[k] = acc;
            }
            __syncthreads();
        }
        // Pass 4: overlaps, hop signs and the H / O accumulation.
        int nanti = 0;
        for (int e = tid; e < 2 * Ns; e += NT) {
            const int4 E = J.edges[e];
            nanti += (s_fock[E.x] >= 0) != (s_fock[E.y] >= 0) ? 1 : 0;
        }
        double wsum = 0.0;
        for (int k = tid; k < Nexc; k += NT) {
            cx<double> a = {1.0, 0.0};
            if (k != cur) a = to_d(s_Y[k]) * to_d(s_g[s_wslot[Ns + s_exd[k]]]);
            s_a[k] = a;
            wsum += norm2(a);
        }
#pragma unroll
        for (int o = 16; o; o >>= 1) {
            nanti += __shfl_xor_sync(0xffffffffu, nanti, o);
            wsum += __shfl_xor_sync(0xffffffffu, wsum, o);
        }
        if (lane == 0) { s_red[warp * 2] = wsum; s_red[warp * 2 + 1] = double(nanti); }
        __syncthreads();
        wsum = 0.0;
        double na = 0.0;
        for (int q = 0; q < NW; ++q) { wsum += s_red[q * 2]; na += s_red[q * 2 + 1]; }
        const double npar = double(2 * Ns) - na;
        // hop signs, one warp per state
        for (int k = warp; k < Nexc; k += NW) {
            int n = 0;
            if (k != cur)
                n = warp_count_between(s_wslot, ocur, s_exu[k]) + warp_count_between(s_wslot + Ns, s_exd[k], hcur);
            if (lane == 0) {
                const double hs = (n & 1) ? -1.0 : 1.0;
                const cx<double> a = s_a[k], S = s_S[k];
                s_hh[k] = cx<double>{hs * (a.x * 0.25 * (npar - na) - 0.5 * S.x), hs * (a.y * 0.25 * (npar - na) - 0.5 * S.y)};
                s_a[k] = cx<double>{hs * a.x, hs * a.y};
            }
        }
        __syncthreads();
        const double iw = 1.0 / wsum;
        cx<double>* H = J.pjx + size_t(w) * 2 * Nexc * Nexc;
        cx<double>* O = H + size_t(Nexc) * Nexc;
        bool narrow = false;
        if constexpr (sizeof(T) == 4) {
            // Mixed form: the Nexc^2 outer products in FP32 (their factors come
            // from FP32 ratios; conj(a_k1) / sum|a|^2 rounded once per state),
            // summed over a block of kHoSlots measurements and then widened
            // into the FP64 sums (ho_push): per measurement 3 Nexc FP32 factors
            // are written instead of the 2 Nexc^2 FP64 sums read and written.
            // A walker whose factors could take a product near the FP32 range
            // (any |factor| > 1e15) adds FP64 products at once.
            cx<float>* s_caf = reinterpret_cast<cx<float>*>(smem + lay.f32);
            cx<float>* s_hf = s_caf + Nexc;
            cx<float>* s_af = s_hf + Nexc;
            bool big = false;
            for (int k = tid; k < Nexc; k += NT) {
                const double m = fmax(fmax(fabs(s_a[k].x), fabs(s_a[k].y)), fmax(fabs(s_hh[k].x), fabs(s_hh[k].y)));
                big = big || !(m <= 1e15) || !(fmax(fabs(s_a[k].x), fabs(s_a[k].y)) * iw <= 1e15);
                s_caf[k] = cx<float>{float(s_a[k].x * iw), float(-s_a[k].y * iw)};
                s_hf[k] = cx<float>{float(s_hh[k].x), float(s_hh[k].y)};
                s_af[k] = cx<float>{float(s_a[k].x), float(s_a[k].y)};
            }
            narrow = !__syncthreads_or(big);
        }
        if (narrow) {
            ho_push<NT>(J, w, reinterpret_cast<const cx<float>*>(smem + lay.f32));
        } else {
            for (int idx = tid; idx < Nexc * Nexc; idx += NT) {
                const int k1 = idx / Nexc, k2 = idx % Nexc;
                const cx<double> ca = {s_a[k1].x, -s_a[k1].y};
                const cx<double> hv = ca * s_hh[k2], ov = ca * s_a[k2];
                H[idx].x += hv.x * iw; H[idx].y += hv.y * iw;
                O[idx].x += ov.x * iw; O[idx].y += ov.y * iw;
            }
        }
        if (tid == 0) J.pj_n[w] += 1;
        __syncthreads();
    }
    if (mask & GV_MEAS_STAGMAGN) {   // StagMagnZ (StagMagnZ.cpp:12-43)
        int m = 0;
        for (int v = tid; v < Ns; v += NT) {
            const int sg = (((v % L) + (v / L)) & 1) ? -1 : 1;
            m += sg * (s_fock[v] >= 0 ? 1 : -1);
        }
#pragma unroll
        for (int o = 16; o; o >>= 1) m += __shfl_xor_sync(0xffffffffu, m, o);
        if (lane == 0) s_red[warp * 2] = double(m);
        __syncthreads();
        if (tid == 0) {
            double t = 0;
            for (int q = 0; q < NW; ++q) t += s_red[q * 2];
            J.sm[w].x += t * inv_ns;
            J.sm_n[w] += 1;
        }
    }
}

// SlaterDeterminant::VirtUpdate (SlaterDeterminant.cpp:96-268) in the
// exciton channel for explicit real-space hop sets of one walker (one block
// per set): out[2*(k*nset + i)] = hs_k rho0_k rho1_k, the ratio qs / Amp()
// of set i and channel state k, from the same formulas as the walk (a
// flavour without a real hop contributes its row-only ratio).
template <typename T, int NT>
__global__ void __launch_bounds__(NT) k_virt_trans(DevJob J, int w, int nset, const int32_t* hops, double* out)
{
    constexpr int NW = NT / 32;
    const int set = blockIdx.x;
    if (set >= nset) return;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int Ns = J.Ns, Nmax = J.Nmax, L = J.L, Nk = J.Nk, Nexc = J.Nexc;
    const int N0 = J.N[0], N1 = J.N[1];
    const int16_t* fock = J.fock + size_t(w) * 2 * Ns;
    const int16_t* wslot = J.wslot + size_t(w) * 2 * Ns;
    const int16_t* worb = J.worb + size_t(w) * 2 * Nmax;
    const cx<T>* phase = Tab<T>::phase(J);
    const cx<T>* cf0 = Tab<T>::coef(J) + size_t(w) * 4 * Ns;
    const cx<T>* cf1 = cf0 + 2 * Ns;
    const cx<T>* A0 = ai_ptr<T>(J, 0, w);
    const cx<T>* A1 = ai_ptr<T>(J, 1, w);
    const cx<T>* G = static_cast<const cx<T>*>(J.gup) + size_t(w) * N0 * Nexc;
    const cx<T>* g = static_cast<const cx<T>*>(J.gdn) + size_t(w) * Nmax;
    extern __shared__ __align__(16) char smem[];
    cx<T>* C0 = reinterpret_cast<cx<T>*>(smem);
    cx<T>* C1 = C0 + Nmax;
    double* red = reinterpret_cast<double*>(C1 + Nmax);
    const int cur = J.cur[w];
    const int ocur = J.exc_up[cur], hcur = J.exc_dn[cur];
    const int r0 = max(int(wslot[ocur]), 0);
    const int uf = hops[4 * set], ut = hops[4 * set + 1], df = hops[4 * set + 2], dt = hops[4 * set + 3];
    const int cu = uf >= 0 ? fock[uf] : -1, cd = df >= 0 ? fock[Ns + df] : -1;
    if ((uf >= 0 && cu < 0) || (df >= 0 && cd < 0)) {   // no particle of that flavour there
        for (int k = tid; k < Nexc; k += NT) { out[2 * (size_t(k) * nset + set)] = nan(""); out[2 * (size_t(k) * nset + set) + 1] = nan(""); }
        return;
    }
    cx<T> m11u = {T(0), T(0)}, m11d = {T(0), T(0)}, gc = {T(0), T(0)};
    if (uf >= 0)
        for (int f = tid; f < N0; f += NT) {
            const cx<T> c = phi_orb<T>(phase, cf0, Nk, Ns, L, ut, worb[f]);
            C0[f] = c;
            cmac(m11u, A0[size_t(f) * N0 + cu], c);
        }
    if (df >= 0)
        for (int f = tid; f < N1; f += NT) {
            const cx<T> c = phi_orb<T>(phase, cf1, Nk, Ns, L, dt, worb[Nmax + f]);
            C1[f] = c;
            cmac(m11d, A1[size_t(f) * N1 + cd], c);
            cmac(gc, g[f], c);
        }
    m11u = warp_sum(m11u);
    m11d = warp_sum(m11d);
    gc = warp_sum(gc);
    if (lane == 0) {
        red[warp * 6 + 0] = double(m11u.x); red[warp * 6 + 1] = double(m11u.y);
        red[warp * 6 + 2] = double(m11d.x); red[warp * 6 + 3] = double(m11d.y);
        red[warp * 6 + 4] = double(gc.x);   red[warp * 6 + 5] = double(gc.y);
    }
    __syncthreads();
    cx<T> M11u = {T(0), T(0)}, M11d = {T(0), T(0)}, gC = {T(0), T(0)};
    for (int q = 0; q < NW; ++q) {
        M11u.x += T(red[q * 6 + 0]); M11u.y += T(red[q * 6 + 1]);
        M11d.x += T(red[q * 6 + 2]); M11d.y += T(red[q * 6 + 3]);
        gC.x += T(red[q * 6 + 4]);   gC.y += T(red[q * 6 + 5]);
    }
    for (int k = tid; k < Nexc; k += NT) {
        cx<T> ru = {T(1), T(0)}, rd = {T(1), T(0)};
        const int rk = wslot[Ns + J.exc_dn[k]];
        if (uf >= 0) {
            ru = M11u;
            if (k != cur) {
                cx<T> Z = {T(0), T(0)};
                for (int f = 0; f < N0; ++f) cmac(Z, G[size_t(f) * Nexc + k], C0[f]);
                ru = M11u * G[size_t(r0) * Nexc + k] -
                     A0[size_t(r0) * N0 + cu] * (Z - phi_orb<T>(phase, cf0, Nk, Ns, L, ut, J.exc_up[k]));
            }
        } else if (k != cur) {
            ru = G[size_t(r0) * Nexc + k];
        }
        if (df >= 0) {
            rd = M11d;
            if (k != cur) rd = M11d * g[rk] - A1[size_t(rk) * N1 + cd] * (gC - phi_orb<T>(phase, cf1, Nk, Ns, L, dt, hcur));
        } else if (k != cur) {
            rd = g[rk];
        }
        int n = 0;
        if (k != cur) {
            for (int x = min(ocur, int(J.exc_up[k])) + 1; x < max(ocur, int(J.exc_up[k])); ++x) n += wslot[x] >= 0;
            for (int x = min(hcur, int(J.exc_dn[k])) + 1; x < max(hcur, int(J.exc_dn[k])); ++x) n += wslot[Ns + x] >= 0;
        }
        cx<double> r = to_d(ru) * to_d(rd);
        if (n & 1) r = cx<double>{-r.x, -r.y};
        out[2 * (size_t(k) * nset + set)] = r.x;
        out[2 * (size_t(k) * nset + set) + 1] = r.y;
    }
}

}  // namespace
}  // namespace gv
