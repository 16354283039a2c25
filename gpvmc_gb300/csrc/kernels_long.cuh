// Engine kernels for the longitudinal-exciton channel (StagFluxLongExciton,
// StagFluxLongExciton.cpp:6-66).  Included by engine.cu after kernels_trans.cuh.
//
// N0 = N1 = N = Ns/2.  State 2fe replaces, in flavour 0, the lower-band
// orbital h = exc_dn[2fe] (the hole at k - q) by the upper-band orbital
// u = exc_up[2fe] = 2fe + 1; state 2fe + 1 does the same in flavour 1; state
// Ns (at q = 0 or (pi, pi)) is the ground state.  From the current state c a
// state k differs, per flavour, by up to two orbital hops (vacated orbitals
// paired with filled ones in ascending order, State::get_hop_path): two in
// one flavour between states of the same kind, one per flavour otherwise.
//
// Per walker and flavour the engine keeps, besides A^-1, the overlap table of
// every orbital with every Slater row,
//     R[f][o] = sum_p phi_o(x_p) (A^-1)(p, f)            (N x Ns)
// (R[.][o] = e_row for an occupied orbital), so that a state's amplitude
// after an exchange (particle c of the flavour moves from s to t) is the
// (1 + n) x (1 + n) determinant of linalg::DetUpdate's capacitance matrix
// (linalg.cpp:107-400) for the column change and the state's n row changes
// (row r_i takes orbital o_i):
//     B00 = M11 = sum_f (A^-1)(c, f) C[f],      C[f] = phi_{worb[f]}(t)
//     B0j = (A^-1)(c, r_j)
//     Bi0 = Z_{o_i} + d_{o_i} M11 - phi_{o_i}(t) - M11 delta_i
//     Bij = R[r_j][o_i] + (d_{o_i} - delta_i) (A^-1)(c, r_j)
// with Z_o = sum_f R[f][o] C[f], d_o = phi_o(t) - phi_o(s) and
// delta_i = C[r_i] - phi_{worb[r_i]}(s); no column change: Bij = R[r_j][o_i].
// An accepted move applies the same rank-(1 + n) Woodbury update as
// linalg::InvUpdate (linalg.cpp:402-573) to A^-1 and carries R along.
#pragma once

#include "kernels_trans.cuh"

namespace gv {
namespace {

// The flavour holding state k's particle-hole pair (2: ground state).
__host__ __device__ __forceinline__ int long_kind(int k, int Ns) { return k < Ns ? (k & 1) : 2; }

// Orbital hops of flavour fl from state c to state k: V[i] -> F[i], i < n.
__host__ __device__ __forceinline__ int long_hops(int c, int k, int fl, const int16_t* exu, const int16_t* exd,
                                                  int Ns, int V[2], int F[2])
{
    const bool ec = long_kind(c, Ns) == fl, ek = long_kind(k, Ns) == fl;
    if (ec && ek) {
        if (c == k) return 0;
        int v0 = exu[c], v1 = exd[k], f0 = exu[k], f1 = exd[c];
        if (v0 > v1) { const int x = v0; v0 = v1; v1 = x; }
        if (f0 > f1) { const int x = f0; f0 = f1; f1 = x; }
        V[0] = v0; V[1] = v1; F[0] = f0; F[1] = f1;
        return 2;
    }
    if (ec) { V[0] = exu[c]; F[0] = exd[c]; return 1; }
    if (ek) { V[0] = exd[k]; F[0] = exu[k]; return 1; }
    return 0;
}

// State::HopSign (State.cpp:86-115) of one flavour's hops from the prefix
// counts pre[x] = occupied orbitals below x: the first hop counts the
// occupied orbitals strictly between its ends, the second counts them with
// the first hop applied.  Returns the parity.
__host__ __device__ __forceinline__ int long_hop_parity(const int16_t* pre, int n, const int V[2], const int F[2])
{
    if (n == 0) return 0;
    int lo = (V[0] < F[0] ? V[0] : F[0]) + 1, hi = V[0] > F[0] ? V[0] : F[0];
    int odd = (hi > lo ? pre[hi] - pre[lo] : 0) & 1;
    if (n > 1) {
        lo = V[1] < F[1] ? V[1] : F[1];
        hi = V[1] > F[1] ? V[1] : F[1];
        int c2 = hi > lo + 1 ? pre[hi] - pre[lo + 1] : 0;
        if (V[0] > lo && V[0] < hi) c2 -= 1;   // vacated by the first hop
        if (F[0] > lo && F[0] < hi) c2 += 1;   // filled by the first hop
        odd ^= c2 & 1;
    }
    return odd;
}

template <typename T>
__device__ __forceinline__ cx<T> det3(const cx<T>* m, int n)   // row-major n x n, n <= 3
{
    if (n == 0) return cx<T>{T(1), T(0)};
    if (n == 1) return m[0];
    if (n == 2) return m[0] * m[3] - m[1] * m[2];
    return m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) + m[2] * (m[3] * m[7] - m[4] * m[6]);
}

// Inverse of an n x n (n <= 3) complex matrix by its adjugate.
template <typename T>
__device__ __forceinline__ void inv3(const cx<T>* m, int n, cx<T>* mi)
{
    const cx<T> id = cinv(det3(m, n));
    if (n == 1) { mi[0] = id; return; }
    if (n == 2) {
        mi[0] = m[3] * id; mi[1] = cneg(m[1]) * id; mi[2] = cneg(m[2]) * id; mi[3] = m[0] * id;
        return;
    }
    mi[0] = (m[4] * m[8] - m[5] * m[7]) * id;
    mi[1] = (m[2] * m[7] - m[1] * m[8]) * id;
    mi[2] = (m[1] * m[5] - m[2] * m[4]) * id;
    mi[3] = (m[5] * m[6] - m[3] * m[8]) * id;
    mi[4] = (m[0] * m[8] - m[2] * m[6]) * id;
    mi[5] = (m[2] * m[3] - m[0] * m[5]) * id;
    mi[6] = (m[3] * m[7] - m[4] * m[6]) * id;
    mi[7] = (m[1] * m[6] - m[0] * m[7]) * id;
    mi[8] = (m[0] * m[4] - m[1] * m[3]) * id;
}

// One flavour's data for evaluating an exchange (shared memory, or global R).
template <typename T>
struct LongFl {
    const cx<T>* rowc;   // (A^-1)(c, f), N
    const cx<T>* del;    // delta_f = C[f] - phi_{worb[f]}(s), N
    const cx<T>* Z;      // Z_o, Ns
    const cx<T>* pt;     // phi_o(t), Ns
    const cx<T>* dd;     // d_o = phi_o(t) - phi_o(s), Ns
    const cx<T>* R;      // R[f][o], N x Ns (global)
    const int16_t* wslot;
    cx<T> M11;
    int Ns;
    bool moved;          // false: no column change (the current configuration)
};

// The capacitance matrix of state k in one flavour (size (moved) + n, row-major),
// returns its size.
template <typename T>
__device__ __forceinline__ int long_cap(const LongFl<T>& D, int n, const int V[2], const int F[2], cx<T>* B)
{
    int r[2];
    for (int i = 0; i < n; ++i) r[i] = max(int(D.wslot[V[i]]), 0);   // V[i] is occupied in the current state
    if (!D.moved) {
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) B[i * n + j] = D.R[size_t(r[j]) * D.Ns + F[i]];
        return n;
    }
    const int m = n + 1;
    B[0] = D.M11;
    for (int j = 0; j < n; ++j) B[1 + j] = D.rowc[r[j]];
    for (int i = 0; i < n; ++i) {
        const int o = F[i];
        const cx<T> di = D.del[r[i]], dm = D.dd[o] - di;
        B[(1 + i) * m] = D.Z[o] + D.dd[o] * D.M11 - D.pt[o] - D.M11 * di;
        for (int j = 0; j < n; ++j) B[(1 + i) * m + 1 + j] = D.R[size_t(r[j]) * D.Ns + o] + dm * D.rowc[r[j]];
    }
    return m;
}

// q_k / Amp of state k (without the wavefunction's hop sign) and, through
// *odd, the parity of that sign.
template <typename T>
__device__ __forceinline__ cx<T> long_state_ratio(const LongFl<T> (&D)[2], int cur, int k, const int16_t* exu,
                                                 const int16_t* exd, const int16_t* pre, int Ns, int* odd)
{
    cx<T> q = {T(1), T(0)};
    int par = 0;
    for (int fl = 0; fl < 2; ++fl) {
        int V[2], F[2];
        const int n = long_hops(cur, k, fl, exu, exd, Ns, V, F);
        cx<T> B[9];
        const int m = long_cap(D[fl], n, V, F, B);
        q = q * det3(B, m);
        par ^= long_hop_parity(pre + fl * (Ns + 1), n, V, F);
    }
    if (odd) *odd = par;
    return q;
}

// Prefix counts of occupied orbitals of both flavours: pre[fl][x] =
// #{o < x : slot[fl][o] >= 0}, x = 0..Ns (one warp per flavour).
__device__ __forceinline__ void long_prefix(const int16_t* wslot, int16_t* pre, int Ns)
{
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp < 2) {
        const int16_t* sl = wslot + warp * Ns;
        int16_t* p = pre + warp * (Ns + 1);
        int base = 0;
        for (int x0 = 0; x0 < Ns; x0 += 32) {
            const int x = x0 + lane;
            int v = (x < Ns && sl[x] >= 0) ? 1 : 0;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, v, o);
                if (lane >= o) v += y;
            }
            if (x < Ns) p[x + 1] = int16_t(base + v);
            base += __shfl_sync(0xffffffffu, v, 31);
        }
        if (lane == 0) p[0] = 0;
    }
}

// Amplitude of every channel state relative to the current one, no move:
// out[w * Nexc + k] = |q_k / Amp|^2 (optional), sigma[w] = the sum (the
// stepper's weight over |Amp|^2, LatticeStepper.cpp:149-169).  One CTA per walker.
template <typename T, int NT>
__global__ void __launch_bounds__(NT) k_long_states(DevJob J, double* out)
{
    extern __shared__ __align__(16) char smem[];
    const int w = blockIdx.x;
    if (w >= J.W || J.status[w] != GV_OK) return;
    const int Ns = J.Ns, Nexc = J.Nexc, tid = threadIdx.x;
    int16_t* s_wslot = reinterpret_cast<int16_t*>(smem);
    int16_t* s_pre = s_wslot + 2 * Ns;
    double* s_red = reinterpret_cast<double*>(smem + ((sizeof(int16_t) * (4 * Ns + 2) + 15) & ~size_t(15)));
    for (int i = tid; i < 2 * Ns; i += NT) s_wslot[i] = J.wslot[size_t(w) * 2 * Ns + i];
    __syncthreads();
    long_prefix(s_wslot, s_pre, Ns);
    __syncthreads();
    LongFl<T> D[2];
    for (int fl = 0; fl < 2; ++fl) {
        D[fl].R = static_cast<const cx<T>*>(J.gup) + (size_t(w) * 2 + fl) * size_t(J.Nmax) * Ns;
        D[fl].wslot = s_wslot + fl * Ns;
        D[fl].Ns = Ns;
        D[fl].moved = false;
    }
    const int cur = J.cur[w];
    double s = 0.0;
    for (int k = tid; k < Nexc; k += NT) {
        const double n = norm2(to_d(long_state_ratio<T>(D, cur, k, J.exc_up, J.exc_dn, s_pre, Ns, nullptr)));
        if (out) out[size_t(w) * Nexc + k] = n;
        s += n;
    }
    s = block_sum_d<NT>(s, s_red);
    if (tid == 0) J.sigma[w] = s;
}

struct LongLayout {
    size_t fock, part, wslot, worb, nbr, exu, exd, pre, coef, rowc, del, C, Z, pt, dd, q, Y, Bi, red, gj, total;
};

template <typename T, int NT>
__host__ __device__ inline LongLayout long_layout(int Ns, int Nmax, int Nexc, bool gj)
{
    LongLayout l;
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
    l.pre = al(sizeof(int16_t) * 2 * (Ns + 1));
    l.coef = al(c * 4 * Ns);
    l.rowc = al(c * 2 * Nmax);
    l.del = al(c * 2 * Nmax);
    l.C = al(c * 2 * Nmax);
    l.Z = al(c * 2 * Ns);
    l.pt = al(c * 2 * Ns);
    l.dd = al(c * 2 * Ns);
    l.q = al(c * Nexc);
    l.Y = al(c * 2 * 3 * Nmax);
    l.Bi = al(c * 2 * 9 + sizeof(int) * 16);
    l.red = al(sizeof(double) * 6 * (NT / 32) + sizeof(int) * (NT / 32) + 64);
    l.gj = al(gj ? gj_smem_bytes(Nmax, NT) : 16);
    l.total = al(16);
    return l;
}

// phi_o(t) and phi_o(t) - phi_o(s) of every orbital of both flavours, for the
// exchange moving flavour 0 from s0 to t0 and flavour 1 from t0 to s0
template <typename T, int NT>
__device__ __forceinline__ void long_stage_phi(const DevJob& J, int s0, int t0, const cx<T>* s_coef, cx<T>* s_pt,
                                               cx<T>* s_dd, bool odd_only = false)
{
    const int tid = threadIdx.x;
    const int Ns = J.Ns, Nk = J.Nk, L = J.L;
    const cx<T>* phase = Tab<T>::phase(J);
    const int nz = odd_only ? Ns : 2 * Ns, per = nz / 2;   // odd_only: the upper-band (odd) orbitals
    for (int idx = tid; idx < nz; idx += NT) {
        const int fl = idx / per, o = odd_only ? 2 * (idx % per) + 1 : idx % Ns;
        const int s = fl ? t0 : s0, t = fl ? s0 : t0;
        const cx<T>* cf = s_coef + fl * 2 * Ns;
        const cx<T> pt = phi_orb<T>(phase, cf, Nk, Ns, L, t, o);
        s_pt[fl * Ns + o] = pt;
        s_dd[fl * Ns + o] = pt - phi_orb<T>(phase, cf, Nk, Ns, L, s, o);
    }
    __syncthreads();
}

// Stage one exchange for both flavours: flavour 0 moves from s0 to t0 and
// flavour 1 from t0 to s0 (rowc, the new column C, delta, phi(t), d, M11,
// and Z; s_Z == nullptr: Z already staged by the caller).  Ends with the CTA
// synchronised and M11 of both flavours in m11[].  zhole < -1: Z over every
// orbital; otherwise only where a state's capacitance matrix reads it: the
// upper-band orbitals (odd, the states' entering orbitals exc_up) of both
// flavours and, when zhole >= 0, the current state's hole zo in flavour zhole.
template <typename T, int NT>
__device__ __forceinline__ void long_stage(const DevJob& J, int w, int s0, int t0, const int16_t* s_fock,
                                           const int16_t* s_worb, const cx<T>* s_coef, cx<T>* s_rowc, cx<T>* s_del,
                                           cx<T>* s_C, cx<T>* s_Z, cx<T>* s_pt, cx<T>* s_dd, double* s_red,
                                           cx<T> m11[2], int zhole = -2, int zo = -1)
{
    constexpr int NW = NT / 32;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int Ns = J.Ns, Nmax = J.Nmax, N = J.N[0], Nk = J.Nk, L = J.L;
    const cx<T>* phase = Tab<T>::phase(J);
    cx<T> acc[2] = {{T(0), T(0)}, {T(0), T(0)}};
    for (int idx = tid; idx < 2 * N; idx += NT) {
        const int fl = idx / N, f = idx % N;
        const int s = fl ? t0 : s0, t = fl ? s0 : t0;
        const int c = max(int(s_fock[fl * Ns + s]), 0);   // the exchange moves a particle of each flavour
        const cx<T>* cf = s_coef + fl * 2 * Ns;
        const int o = s_worb[fl * Nmax + f];
        const cx<T> a = ai_ptr<T>(J, fl, w)[size_t(f) * N + c];
        const cx<T> C = phi_orb<T>(phase, cf, Nk, Ns, L, t, o);
        s_rowc[fl * Nmax + f] = a;
        s_del[fl * Nmax + f] = C - phi_orb<T>(phase, cf, Nk, Ns, L, s, o);
        cmac(acc[fl], a, C);
        s_C[fl * Nmax + f] = C;
    }
    for (int i = 0; i < 2; ++i) acc[i] = warp_sum(acc[i]);
    if (lane == 0) {
        s_red[warp * 4 + 0] = double(acc[0].x); s_red[warp * 4 + 1] = double(acc[0].y);
        s_red[warp * 4 + 2] = double(acc[1].x); s_red[warp * 4 + 3] = double(acc[1].y);
    }
    __syncthreads();
    for (int i = 0; i < 2; ++i) {
        cx<T> m = {T(0), T(0)};
        for (int q = 0; q < NW; ++q) { m.x += T(s_red[q * 4 + 2 * i]); m.y += T(s_red[q * 4 + 2 * i + 1]); }
        m11[i] = m;
    }
    if (s_Z == nullptr) {   // Z staged by the caller (batched bonds): the orbital rows only
        long_stage_phi<T, NT>(J, s0, t0, s_coef, s_pt, s_dd);
        return;
    }
    // Z_o = sum_f R[f][o] C[f] for every orbital of both flavours (or the odd ones)
    const bool sel = zhole >= -1;
    const int nz = sel ? Ns : 2 * Ns, per = nz / 2;
    for (int idx = tid; idx < nz; idx += NT) {
        const int fl = idx / per, o = sel ? 2 * (idx % per) + 1 : idx % Ns;
        const cx<T>* R = static_cast<const cx<T>*>(J.gup) + (size_t(w) * 2 + fl) * size_t(Nmax) * Ns;
        const cx<T>* C = s_C + fl * Nmax;
        cx<T> z = {T(0), T(0)};
        int f = 0;
        for (; f + 4 <= N; f += 4) {
            cx<T> r[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) r[q] = R[size_t(f + q) * Ns + o];
#pragma unroll
            for (int q = 0; q < 4; ++q) cmac(z, r[q], C[f + q]);
        }
        for (; f < N; ++f) cmac(z, R[size_t(f) * Ns + o], C[f]);
        s_Z[fl * Ns + o] = z;
    }
    if (zhole >= 0 && warp == NW - 1) {   // the current hole's sum, split over a warp's lanes
        const cx<T>* R = static_cast<const cx<T>*>(J.gup) + (size_t(w) * 2 + zhole) * size_t(Nmax) * Ns;
        const cx<T>* C = s_C + zhole * Nmax;
        cx<T> z = {T(0), T(0)};
        for (int f = lane; f < N; f += 32) cmac(z, R[size_t(f) * Ns + zo], C[f]);
        z = warp_sum(z);
        if (lane == 0) {
            s_Z[zhole * Ns + zo] = z;
            // and the hole's orbital rows (the odd ones come from long_stage_phi)
            const int s = zhole ? t0 : s0, t = zhole ? s0 : t0;
            const cx<T>* cf = s_coef + zhole * 2 * Ns;
            const cx<T> pt = phi_orb<T>(phase, cf, Nk, Ns, L, t, zo);
            s_pt[zhole * Ns + zo] = pt;
            s_dd[zhole * Ns + zo] = pt - phi_orb<T>(phase, cf, Nk, Ns, L, s, zo);
        }
    }
    __syncthreads();
    long_stage_phi<T, NT>(J, s0, t0, s_coef, s_pt, s_dd, sel);
}

// ------------------------------------------------------------------------
// Metropolis walk, longitudinal-exciton channel: one CTA per walker,
// MetroMC::Step with LatticeStepper::trystep / step (LatticeStepper.cpp:36-147):
// the proposal's weight is the sum over all channel states, the accepted
// move hops the wavefunction to the first arg-max state.
template <typename T, int NT>
__global__ void __launch_bounds__(NT) k_walk_long(DevJob J, uint64_t nsteps, int inkernel_reinv)
{
    extern __shared__ __align__(16) char smem[];
    constexpr int NW = NT / 32;
    const int w = blockIdx.x;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (w >= J.W || J.status[w] != GV_OK) return;
    const bool forced = J.forced_walker >= 0;
    if (forced && w != J.forced_walker) return;
    const int Ns = J.Ns, Nmax = J.Nmax, Nexc = J.Nexc, N = J.N[0];
    const LongLayout lay = long_layout<T, NT>(Ns, Nmax, Nexc, inkernel_reinv != 0);
    int16_t* s_fock = reinterpret_cast<int16_t*>(smem + lay.fock);
    int16_t* s_part = reinterpret_cast<int16_t*>(smem + lay.part);
    int16_t* s_wslot = reinterpret_cast<int16_t*>(smem + lay.wslot);
    int16_t* s_worb = reinterpret_cast<int16_t*>(smem + lay.worb);
    int16_t* s_nbr = reinterpret_cast<int16_t*>(smem + lay.nbr);
    int16_t* s_exu = reinterpret_cast<int16_t*>(smem + lay.exu);
    int16_t* s_exd = reinterpret_cast<int16_t*>(smem + lay.exd);
    int16_t* s_pre = reinterpret_cast<int16_t*>(smem + lay.pre);
    cx<T>* s_coef = reinterpret_cast<cx<T>*>(smem + lay.coef);
    cx<T>* s_rowc = reinterpret_cast<cx<T>*>(smem + lay.rowc);
    cx<T>* s_del = reinterpret_cast<cx<T>*>(smem + lay.del);
    cx<T>* s_C = reinterpret_cast<cx<T>*>(smem + lay.C);
    cx<T>* s_Z = reinterpret_cast<cx<T>*>(smem + lay.Z);
    cx<T>* s_pt = reinterpret_cast<cx<T>*>(smem + lay.pt);
    cx<T>* s_dd = reinterpret_cast<cx<T>*>(smem + lay.dd);
    cx<T>* s_q = reinterpret_cast<cx<T>*>(smem + lay.q);
    cx<T>* s_Y = reinterpret_cast<cx<T>*>(smem + lay.Y);     // [fl][b][f]
    cx<T>* s_Bi = reinterpret_cast<cx<T>*>(smem + lay.Bi);   // [fl][9]
    int* s_hop = reinterpret_cast<int*>(s_Bi + 18);          // [fl]: n, r0, r1, o0, o1, m; [12] parity, [13 + fl] singular
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
    __syncthreads();
    long_prefix(s_wslot, s_pre, Ns);
    __syncthreads();

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
    LongFl<T> D[2];
    for (int fl = 0; fl < 2; ++fl) {
        D[fl].rowc = s_rowc + fl * Nmax;
        D[fl].del = s_del + fl * Nmax;
        D[fl].Z = s_Z + fl * Ns;
        D[fl].pt = s_pt + fl * Ns;
        D[fl].dd = s_dd + fl * Ns;
        D[fl].R = static_cast<const cx<T>*>(J.gup) + (size_t(w) * 2 + fl) * size_t(Nmax) * Ns;
        D[fl].wslot = s_wslot + fl * Ns;
        D[fl].Ns = Ns;
        D[fl].moved = true;
    }

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
            const int s0 = (f1 == 0) ? v1 : v2, t0 = (f1 == 0) ? v2 : v1;
            cx<T> m11[2];
            // Z where the states read it: the odd orbitals, and the current hole in
            // the flavour holding the current pair (the update below forms the rest)
            const int hk = long_kind(cur, Ns);
            const int zhole = hk < 2 ? hk : -1, zo = hk < 2 ? int(s_exd[cur]) : -1;
            long_stage<T, NT>(J, w, s0, t0, s_fock, s_worb, s_coef, s_rowc, s_del, s_C, s_Z, s_pt, s_dd, s_red, m11,
                              zhole, zo);
            D[0].M11 = m11[0];
            D[1].M11 = m11[1];
            // every state's amplitude after the exchange, their weight sum and first arg-max
            T wsum = T(0), wbest = T(-1);
            int kbest = Nexc;
            for (int k = tid; k < Nexc; k += NT) {
                const cx<T> q = long_state_ratio<T>(D, cur, k, s_exu, s_exd, s_pre, Ns, nullptr);
                s_q[k] = q;
                const T wk = norm2(q);
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
            double* rb = s_red + 4 * NW;
            int* rbi = reinterpret_cast<int*>(rb + 2 * NW);
            if (lane == 0) { rb[2 * warp] = double(wsum); rb[2 * warp + 1] = double(wbest); rbi[warp] = kbest; }
            __syncthreads();
            double ws = 0.0, wb = -1.0;
            kbest = Nexc;
            for (int q = 0; q < NW; ++q) {
                ws += rb[2 * q];
                if (rb[2 * q + 1] > wb || (rb[2 * q + 1] == wb && rbi[q] < kbest)) { wb = rb[2 * q + 1]; kbest = rbi[q]; }
            }
            __syncthreads();   // rb is reused by the next step
            khop = (forced && J.forced_khop >= 0 && J.forced_khop < Nexc) ? J.forced_khop : kbest;
            ratio = T(ws / sigma);
            if (!isfinite(ratio) || khop >= Nexc) { status = GV_ERR_NAN; break; }
            accepted = forced ? J.forced_accept : (ratio > T(1) ? 1 : (Accept<T>::uniform(m4) < ratio));
            if (!accepted) {
                ++c_rej;
            } else {
                const cx<T> qk = s_q[khop];
                // capacitance inverse and Y rows of both flavours for state khop
                if (tid < 2) {
                    const int fl = tid;
                    int V[2], F[2];
                    const int n = long_hops(cur, khop, fl, s_exu, s_exd, Ns, V, F);
                    cx<T> B[9];
                    const int m = long_cap<T>(D[fl], n, V, F, B);
                    inv3<T>(B, m, s_Bi + 9 * fl);
                    int* h = s_hop + 6 * fl;
                    h[0] = n; h[5] = m;
                    // a vanishing capacitance determinant is a singular update (linalg.cpp:562-570)
                    s_hop[13 + fl] = !(norm2(det3(B, m)) >= T(1e-9));
                    for (int i = 0; i < n; ++i) { h[1 + i] = max(int(s_wslot[fl * Ns + V[i]]), 0); h[3 + i] = F[i]; }
                }
                __syncthreads();
                if (s_hop[13] || s_hop[14]) { status = GV_ERR_SINGULAR; break; }
                for (int idx = tid; idx < 2 * N; idx += NT) {
                    const int fl = idx / N, f = idx % N;
                    const int* h = s_hop + 6 * fl;
                    const cx<T>* R = D[fl].R;
                    const cx<T> rc = s_rowc[fl * Nmax + f];
                    cx<T>* Y = s_Y + fl * 3 * Nmax;
                    Y[f] = rc;
                    for (int i = 0; i < h[0]; ++i) {
                        const int ri = h[1 + i], o = h[3 + i];
                        cx<T> v = R[size_t(f) * Ns + o] + (s_dd[fl * Ns + o] - s_del[fl * Nmax + ri]) * rc;
                        if (f == ri) v.x -= T(1);
                        Y[(1 + i) * Nmax + f] = v;
                    }
                }
                __syncthreads();
                // A^-1 <- A^-1 - X B^-1 Y, column p per thread: X[p] = (w_p - [p == c], A^-1(p, r_j))
                for (int idx = tid; idx < 2 * N; idx += NT) {
                    const int fl = idx / N, p = idx % N;
                    const int* h = s_hop + 6 * fl;
                    const int m = h[5];
                    cx<T>* A = ai_ptr<T>(J, fl, w);
                    const int s = fl ? t0 : s0;
                    const int c = s_fock[fl * Ns + s];
                    cx<T> X[3];
                    X[0] = col_dot<T>(A, N, p, s_C + fl * Nmax);   // w_p = (A^-1 C)_p
                    if (p == c) X[0].x -= T(1);
                    for (int j = 0; j < h[0]; ++j) X[1 + j] = A[size_t(h[1 + j]) * N + p];
                    const cx<T>* Bi = s_Bi + 9 * fl;
                    cx<T> al[3];
                    for (int b = 0; b < m; ++b) {
                        al[b] = cx<T>{T(0), T(0)};
                        for (int a = 0; a < m; ++a) cmac(al[b], X[a], Bi[a * m + b]);
                    }
                    const cx<T>* Y = s_Y + fl * 3 * Nmax;
                    for (int f = 0; f < N; ++f) {
                        cx<T> v = A[size_t(f) * N + p];
                        for (int b = 0; b < m; ++b) cmac(v, cneg(al[b]), Y[b * Nmax + f]);
                        A[size_t(f) * N + p] = v;
                    }
                }
                // R <- R + (A^-1(c, .)) d^T - (Xo B^-1 Y)^T, orbital column o per thread:
                // Xo[o] = (Z_o + d_o M11 - phi_o(t), R[r_j][o] + d_o A^-1(c, r_j))
                for (int idx = tid; idx < 2 * Ns; idx += NT) {
                    const int fl = idx / Ns, o = idx % Ns;
                    const int* h = s_hop + 6 * fl;
                    const int m = h[5];
                    cx<T>* R = static_cast<cx<T>*>(J.gup) + (size_t(w) * 2 + fl) * size_t(Nmax) * Ns;
                    cx<T> d = s_dd[fl * Ns + o], ptv = s_pt[fl * Ns + o];
                    cx<T> zv = s_Z[fl * Ns + o];
                    if (!(o & 1) && !(fl == zhole && o == zo)) {   // an orbital the staging left out
                        const int sf = fl ? t0 : s0, tf = fl ? s0 : t0;
                        const cx<T>* cfo = s_coef + fl * 2 * Ns;
                        ptv = phi_orb<T>(Tab<T>::phase(J), cfo, J.Nk, Ns, J.L, tf, o);
                        d = ptv - phi_orb<T>(Tab<T>::phase(J), cfo, J.Nk, Ns, J.L, sf, o);
                        const cx<T>* C = s_C + fl * Nmax;
                        zv = cx<T>{T(0), T(0)};
                        int f = 0;
                        for (; f + 4 <= N; f += 4) {
                            cx<T> r[4];
#pragma unroll
                            for (int q = 0; q < 4; ++q) r[q] = R[size_t(f + q) * Ns + o];
#pragma unroll
                            for (int q = 0; q < 4; ++q) cmac(zv, r[q], C[f + q]);
                        }
                        for (; f < N; ++f) cmac(zv, R[size_t(f) * Ns + o], C[f]);
                    }
                    cx<T> X[3];
                    X[0] = zv + d * D[fl].M11 - ptv;
                    for (int j = 0; j < h[0]; ++j) X[1 + j] = R[size_t(h[1 + j]) * Ns + o] + d * s_rowc[fl * Nmax + h[1 + j]];
                    const cx<T>* Bi = s_Bi + 9 * fl;
                    cx<T> be[3];
                    for (int b = 0; b < m; ++b) {
                        be[b] = cx<T>{T(0), T(0)};
                        for (int a = 0; a < m; ++a) cmac(be[b], X[a], Bi[a * m + b]);
                    }
                    const cx<T>* Y = s_Y + fl * 3 * Nmax;
                    for (int f = 0; f < N; ++f) {
                        cx<T> v = R[size_t(f) * Ns + o];
                        cmac(v, s_rowc[fl * Nmax + f], d);
                        for (int b = 0; b < m; ++b) cmac(v, cneg(be[b]), Y[b * Nmax + f]);
                        R[size_t(f) * Ns + o] = v;
                    }
                }
                __syncthreads();
                int odd = 0;
                if (tid == 0) {
                    const int cu = s_fock[s0], cd = s_fock[Ns + t0];
                    s_fock[t0] = int16_t(cu); s_fock[s0] = -1; s_part[cu] = int16_t(t0);
                    s_fock[Ns + s0] = int16_t(cd); s_fock[Ns + t0] = -1; s_part[Nmax + cd] = int16_t(s0);
                    // WaveFunction::Hop to khop: rows keep their index and change orbital
                    for (int fl = 0; fl < 2; ++fl) {
                        int V[2], F[2];
                        const int n = long_hops(cur, khop, fl, s_exu, s_exd, Ns, V, F);
                        odd ^= long_hop_parity(s_pre + fl * (Ns + 1), n, V, F);
                        for (int i = 0; i < n; ++i) {
                            const int r = max(int(s_wslot[fl * Ns + V[i]]), 0);
                            s_wslot[fl * Ns + V[i]] = -1;
                            s_wslot[fl * Ns + F[i]] = int16_t(r);
                            s_worb[fl * Nmax + r] = int16_t(F[i]);
                        }
                    }
                    am = am * to_d(qk);
                    amp_normalise(am, ae);
                    s_hop[12] = odd;
                }
                __syncthreads();
                wsign *= s_hop[12] ? -1 : 1;
                cur = khop;
                sigma = ws / double(norm2(qk));
                long_prefix(s_wslot, s_pre, Ns);
                ++c_acc;
                ++since;
                __syncthreads();
                if (inkernel_reinv && J.reinv_every > 0 && since >= J.reinv_every) {
                    char* gp = smem + lay.gj;
                    GJSmem GS = carve_gj<NT>(gp, Nmax);
                    cx<double>* M = J.scratch64 + size_t(w) * Nmax * Nmax;
                    const int st = reinvert_walker<T, NT>(J, w, M, GS, s_part, s_worb);
                    if (st != GV_OK) { status = st; break; }
                    long_rebuild<T, NT>(J, w, s_part);
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
    if (tid == 0) {
        if (!forced) J.rng_next[w] = kk;
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

// Shared-memory pieces of the measurement and VirtUpdate kernels.
constexpr int kLongBonds = 8;   // bonds whose overlap sums Z share one pass over R in a measurement
constexpr int kLongZBonds = 4;  // bonds staged together when the sums come from the tensor cores

struct LongMeasLayout {
    size_t fock, part, wslot, worb, exu, exd, pre, coef, rowc, del, C, Z, pt, dd, S, a, hh, f32, bl, Cb, Zb, red, total;
};

template <typename T, int NT>
__host__ __device__ inline LongMeasLayout long_meas_layout(int Ns, int Nmax, int Nexc)
{
    LongMeasLayout l;
    size_t b = 0;
    auto al = [&](size_t x) { b = (b + 15) & ~size_t(15); size_t r = b; b += x; return r; };
    const size_t c = sizeof(cx<T>);
    l.fock = al(sizeof(int16_t) * 2 * Ns);
    l.part = al(sizeof(int16_t) * 2 * Nmax);
    l.wslot = al(sizeof(int16_t) * 2 * Ns);
    l.worb = al(sizeof(int16_t) * 2 * Nmax);
    l.exu = al(sizeof(int16_t) * Nexc);
    l.exd = al(sizeof(int16_t) * Nexc);
    l.pre = al(sizeof(int16_t) * 2 * (Ns + 1));
    l.coef = al(c * 4 * Ns);
    l.rowc = al(c * 2 * Nmax);
    l.del = al(c * 2 * Nmax);
    l.C = al(c * 2 * Nmax);
    l.Z = al(c * 2 * Ns);
    l.pt = al(c * 2 * Ns);
    l.dd = al(c * 2 * Ns);
    l.S = al(sizeof(cx<double>) * Nexc);
    l.a = al(sizeof(cx<double>) * Nexc);
    l.hh = al(sizeof(cx<double>) * Nexc);
    l.f32 = l.Z;   // FP32 factors of the H / O outer products (mixed form): over Z, pt, dd, dead by then
    l.bl = al(sizeof(int32_t) * 2 * Ns);                    // antiparallel bonds (s0 | t0 << 16), creation order
    l.Cb = al(c * kLongBonds * 2 * Nmax);                   // [bond][fl][f] new columns of a batch of bonds
    l.Zb = al(c * kLongBonds * 2 * Ns);                     // [bond][fl][o] their overlap sums
    l.red = al(sizeof(double) * 4 * (NT / 32) + 64);
    l.total = al(16);
    return l;
}

template <typename T, int NT>
__device__ __forceinline__ void long_load(const DevJob& J, int w, const LongMeasLayout& lay, char* smem)
{
    const int Ns = J.Ns, Nmax = J.Nmax, Nexc = J.Nexc, tid = threadIdx.x;
    int16_t* s_fock = reinterpret_cast<int16_t*>(smem + lay.fock);
    int16_t* s_part = reinterpret_cast<int16_t*>(smem + lay.part);
    int16_t* s_wslot = reinterpret_cast<int16_t*>(smem + lay.wslot);
    int16_t* s_worb = reinterpret_cast<int16_t*>(smem + lay.worb);
    int16_t* s_exu = reinterpret_cast<int16_t*>(smem + lay.exu);
    int16_t* s_exd = reinterpret_cast<int16_t*>(smem + lay.exd);
    cx<T>* s_coef = reinterpret_cast<cx<T>*>(smem + lay.coef);
    for (int i = tid; i < 2 * Ns; i += NT) {
        s_fock[i] = J.fock[size_t(w) * 2 * Ns + i];
        s_wslot[i] = J.wslot[size_t(w) * 2 * Ns + i];
    }
    for (int i = tid; i < 2 * Nmax; i += NT) {
        s_part[i] = J.part[size_t(w) * 2 * Nmax + i];
        s_worb[i] = J.worb[size_t(w) * 2 * Nmax + i];
    }
    for (int i = tid; i < Nexc; i += NT) { s_exu[i] = J.exc_up[i]; s_exd[i] = J.exc_dn[i]; }
    const cx<T>* cg = Tab<T>::coef(J) + size_t(w) * 4 * Ns;
    for (int i = tid; i < 4 * Ns; i += NT) s_coef[i] = cg[i];
    __syncthreads();
    long_prefix(s_wslot, reinterpret_cast<int16_t*>(smem + lay.pre), Ns);
    __syncthreads();
}

// ProjHeis (ProjHeis.cpp:40-158) and StagMagnZ (StagMagnZ.cpp:12-43) in the
// longitudinal channel, one CTA per walker: a_k = q_k / Amp for every state
// (no move), S_k = sum over antiparallel bonds of q_k(bond) / Amp, and
//     h_k = a_k (npar - nanti) / 4 - S_k / 2,
//     H[k1][k2] += conj(a_k1) h_k2 / w,  O[k1][k2] += conj(a_k1) a_k2 / w,
// w = sum_k |a_k|^2, as the transverse channel's measurement.
//
// zpre (mixed form, or null): the bonds' overlap sums Z[w][fl][b][o] from the
// tensor cores (k_long_z_tc), in place of the sums formed here from R.
template <typename T, int NT>
__global__ void __launch_bounds__(NT) k_measure_long(DevJob J, int mask, const cx<float>* zpre)
{
    extern __shared__ __align__(16) char smem[];
    constexpr int NW = NT / 32;
    const int w = blockIdx.x;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (w >= J.W || J.status[w] != GV_OK) return;
    const int Ns = J.Ns, Nmax = J.Nmax, Nexc = J.Nexc, L = J.L;
    const LongMeasLayout lay = long_meas_layout<T, NT>(Ns, Nmax, Nexc);
    long_load<T, NT>(J, w, lay, smem);
    const int16_t* s_fock = reinterpret_cast<const int16_t*>(smem + lay.fock);
    const int16_t* s_wslot = reinterpret_cast<const int16_t*>(smem + lay.wslot);
    const int16_t* s_worb = reinterpret_cast<const int16_t*>(smem + lay.worb);
    const int16_t* s_exu = reinterpret_cast<const int16_t*>(smem + lay.exu);
    const int16_t* s_exd = reinterpret_cast<const int16_t*>(smem + lay.exd);
    const int16_t* s_pre = reinterpret_cast<const int16_t*>(smem + lay.pre);
    const cx<T>* s_coef = reinterpret_cast<const cx<T>*>(smem + lay.coef);
    cx<T>* s_rowc = reinterpret_cast<cx<T>*>(smem + lay.rowc);
    cx<T>* s_del = reinterpret_cast<cx<T>*>(smem + lay.del);
    cx<T>* s_C = reinterpret_cast<cx<T>*>(smem + lay.C);
    cx<T>* s_Z = reinterpret_cast<cx<T>*>(smem + lay.Z);
    cx<T>* s_pt = reinterpret_cast<cx<T>*>(smem + lay.pt);
    cx<T>* s_dd = reinterpret_cast<cx<T>*>(smem + lay.dd);
    cx<double>* s_S = reinterpret_cast<cx<double>*>(smem + lay.S);
    cx<double>* s_a = reinterpret_cast<cx<double>*>(smem + lay.a);
    cx<double>* s_hh = reinterpret_cast<cx<double>*>(smem + lay.hh);
    double* s_red = reinterpret_cast<double*>(smem + lay.red);
    const int cur = J.cur[w];
    LongFl<T> D[2];
    for (int fl = 0; fl < 2; ++fl) {
        D[fl].rowc = s_rowc + fl * Nmax;
        D[fl].del = s_del + fl * Nmax;
        D[fl].Z = s_Z + fl * Ns;
        D[fl].pt = s_pt + fl * Ns;
        D[fl].dd = s_dd + fl * Ns;
        D[fl].R = static_cast<const cx<T>*>(J.gup) + (size_t(w) * 2 + fl) * size_t(Nmax) * Ns;
        D[fl].wslot = s_wslot + fl * Ns;
        D[fl].Ns = Ns;
        D[fl].moved = false;
    }
    if (mask & GV_MEAS_PROJHEIS) {
        double wsum = 0.0;
        for (int k = tid; k < Nexc; k += NT) {
            const cx<double> a = to_d(long_state_ratio<T>(D, cur, k, s_exu, s_exd, s_pre, Ns, nullptr));
            s_a[k] = a;
            s_S[k] = cx<double>{0.0, 0.0};
            wsum += norm2(a);
        }
        wsum = block_sum_d<NT>(wsum, s_red);
        D[0].moved = D[1].moved = true;
        // The antiparallel bonds in creation order (SquareLattice.cpp:9-28),
        // compacted: each warp ballots its 32 bonds, the warps' counts are
        // prefix-summed in shared memory.
        int32_t* s_bl = reinterpret_cast<int32_t*>(smem + lay.bl);
        int* s_cnt = reinterpret_cast<int*>(s_red);
        int nanti = 0;
        for (int e0 = 0; e0 < 2 * Ns; e0 += NT) {
            const int e = e0 + tid;
            bool anti = false;
            int code = 0;
            if (e < 2 * Ns) {
                const int4 E = J.edges[e];
                const bool ua = s_fock[E.x] >= 0, ub = s_fock[E.y] >= 0;
                anti = ua != ub;
                code = ua ? (E.x | (E.y << 16)) : (E.y | (E.x << 16));   // s0 | t0 << 16
            }
            const unsigned bal = __ballot_sync(0xffffffffu, anti);
            if (lane == 0) s_cnt[warp] = __popc(bal);
            __syncthreads();
            int off = nanti, tot = 0;
            for (int q = 0; q < NW; ++q) {
                if (q < warp) off += s_cnt[q];
                tot += s_cnt[q];
            }
            if (anti) s_bl[off + __popc(bal & ((1u << lane) - 1u))] = code;
            nanti += tot;
            __syncthreads();
        }
        cx<T>* s_Cb = reinterpret_cast<cx<T>*>(smem + lay.Cb);
        cx<T>* s_Zb = reinterpret_cast<cx<T>*>(smem + lay.Zb);
        const int N = J.N[0], Nk = J.Nk;
        const cx<T>* phase = Tab<T>::phase(J);
        bool zt = false;   // Z of every bond precomputed
        if constexpr (sizeof(T) == 4) {
            zt = zpre != nullptr;
            if (zt) {
                // Bonds in batches of kLongZBonds: per batch one staging pass
                // (Z rows copied in, phi_o(t) and phi_o(t) - phi_o(s) of every
                // orbital, the moving particles' inverse rows and M11 with a
                // warp per bond and flavour), one barrier, then every state's
                // ratio for every bond of the batch.  The batch arrays reuse the
                // buffers of the per-bond form: Z and phi(t) rows over Zb,
                // phi(t) - phi(s) over Cb, inverse rows and deltas over
                // rowc .. dd (contiguous), M11 over the reduction scratch.
                constexpr int NBZ = kLongZBonds;
                // the states read Z, phi(t) and phi(t) - phi(s) only at the orbitals
                // they enter: the upper-band orbitals (odd) and the current hole
                const int Nh = Ns / 2;
                const int hk = long_kind(cur, Ns);
                const int zhole = hk < 2 ? hk : -1, zo = hk < 2 ? int(s_exd[cur]) : -1;
                cx<float>* ZB = s_Zb;
                cx<float>* ptB = s_Zb + NBZ * 2 * Ns;
                cx<float>* ddB = s_Cb;
                cx<float>* rowcB = s_rowc;
                cx<float>* delB = s_rowc + NBZ * 2 * Nmax;
                cx<float>* m11B = reinterpret_cast<cx<float>*>(s_red);   // 2 NBZ values (64 B)
                // the ratios of the states past the block's threads (Nexc <= Ns + 1 <= NT + 1
                // here, so at most NBZ values) before they are added in bond order
                cx<double>* xq = reinterpret_cast<cx<double>*>(s_red + 16);
                for (int b0 = 0; b0 < nanti; b0 += NBZ) {
                    const int nb = nanti - b0 < NBZ ? nanti - b0 : NBZ;
                    for (int idx = tid; idx < nb * 2 * (Nh + 1); idx += NT) {
                        const int j = idx / (2 * (Nh + 1)), fl = (idx / (Nh + 1)) & 1, r = idx % (Nh + 1);
                        if (r == Nh && fl != zhole) continue;   // no hole in this flavour
                        const int o = r < Nh ? 2 * r + 1 : zo;
                        const int code = s_bl[b0 + j], s0 = code & 0xFFFF, t0 = code >> 16;
                        const int sf = fl ? t0 : s0, tf = fl ? s0 : t0;
                        const cx<float>* cf = s_coef + fl * 2 * Ns;
                        const int e = (j * 2 + fl) * Ns + o;
                        if (r < Nh) ZB[e] = zpre[((size_t(w) * 2 + fl) * 2 * Ns + (b0 + j)) * Nh + r];
                        const cx<float> pt = phi_orb<float>(phase, cf, Nk, Ns, L, tf, o);
                        ptB[e] = pt;
                        ddB[e] = pt - phi_orb<float>(phase, cf, Nk, Ns, L, sf, o);
                    }
                    for (int seg = warp; seg < nb * 2; seg += NW) {
                        const int j = seg >> 1, fl = seg & 1;
                        const int code = s_bl[b0 + j], s0 = code & 0xFFFF, t0 = code >> 16;
                        const int sf = fl ? t0 : s0, tf = fl ? s0 : t0;
                        const int c = max(int(s_fock[fl * Ns + sf]), 0);   // the exchange moves a particle of each flavour
                        const cx<float>* cf = s_coef + fl * 2 * Ns;
                        const cx<float>* ai = ai_ptr<float>(J, fl, w);
                        const cx<float>* Rh = fl == zhole ? D[fl].R + zo : nullptr;   // the hole's column of R
                        cx<float> acc = {0.f, 0.f}, zh = {0.f, 0.f};
                        for (int f = lane; f < N; f += 32) {
                            const int o = s_worb[fl * Nmax + f];
                            const cx<float> a = ai[size_t(f) * N + c];
                            const cx<float> C = phi_orb<float>(phase, cf, Nk, Ns, L, tf, o);
                            rowcB[seg * Nmax + f] = a;
                            delB[seg * Nmax + f] = C - phi_orb<float>(phase, cf, Nk, Ns, L, sf, o);
                            cmac(acc, a, C);
                            if (Rh) cmac(zh, Rh[size_t(f) * Ns], C);
                        }
                        acc = warp_sum(acc);
                        if (lane == 0) m11B[seg] = acc;
                        if (Rh) {   // Z at the hole, which the tensor-core sums leave out
                            zh = warp_sum(zh);
                            if (lane == 0) ZB[seg * Ns + zo] = zh;
                        }
                    }
                    __syncthreads();
                    // the bond's view of both flavours for state evaluations
                    auto bond_view = [&](int jb, LongFl<float> (&Dj)[2]) {
                        Dj[0] = D[0];
                        Dj[1] = D[1];
                        for (int fl = 0; fl < 2; ++fl) {
                            const int seg = jb * 2 + fl;
                            Dj[fl].rowc = rowcB + seg * Nmax;
                            Dj[fl].del = delB + seg * Nmax;
                            Dj[fl].Z = ZB + seg * Ns;
                            Dj[fl].pt = ptB + seg * Ns;
                            Dj[fl].dd = ddB + seg * Ns;
                            Dj[fl].M11 = m11B[seg];
                            Dj[fl].moved = true;
                        }
                    };
                    // one state per thread for every bond of the batch; the states past
                    // the block's threads (the ground state, Nexc = Ns + 1) one
                    // (state, bond) pair per thread, so that no thread takes two states
                    const int k1 = Nexc < NT ? Nexc : NT;
                    for (int k = tid; k < k1; k += NT) {
                        cx<double> sk = {0.0, 0.0};
                        for (int jb = 0; jb < nb; ++jb) {
                            LongFl<float> Dj[2];
                            bond_view(jb, Dj);
                            const cx<double> q = to_d(long_state_ratio<float>(Dj, cur, k, s_exu, s_exd, s_pre, Ns, nullptr));
                            sk.x += q.x;
                            sk.y += q.y;
                        }
                        s_S[k].x += sk.x;
                        s_S[k].y += sk.y;
                    }
                    for (int pq = tid; pq < (Nexc - k1) * nb; pq += NT) {   // into xq, added in bond order below
                        const int k = k1 + pq / nb, jb = pq % nb;
                        LongFl<float> Dj[2];
                        bond_view(jb, Dj);
                        xq[pq] = to_d(long_state_ratio<float>(Dj, cur, k, s_exu, s_exd, s_pre, Ns, nullptr));
                    }
                    __syncthreads();   // the next batch restages
                    if (tid == 0)
                        for (int k = k1; k < Nexc; ++k)
                            for (int jb = 0; jb < nb; ++jb) {
                                s_S[k].x += xq[(k - k1) * nb + jb].x;
                                s_S[k].y += xq[(k - k1) * nb + jb].y;
                            }
                }
                __syncthreads();   // every state's bond sums are in s_S
            }
        }
        for (int b0 = 0; !zt && b0 < nanti; b0 += kLongBonds) {
            const int nb = nanti - b0 < kLongBonds ? nanti - b0 : kLongBonds;
            // the new columns C of the batch's bonds (as long_stage forms them)
            for (int idx = tid; idx < nb * 2 * N; idx += NT) {
                const int j = idx / (2 * N), fl = (idx / N) & 1, f = idx % N;
                const int code = s_bl[b0 + j], s0 = code & 0xFFFF, t0 = code >> 16;
                const int t = fl ? s0 : t0;
                s_Cb[(j * 2 + fl) * Nmax + f] = phi_orb<T>(phase, s_coef + fl * 2 * Ns, Nk, Ns, L, t, s_worb[fl * Nmax + f]);
            }
            __syncthreads();
            // Z_o = sum_f R[f][o] C[f] of every bond of the batch in one pass over R
            // (each sum in the order long_stage takes it)
            for (int idx = tid; idx < 2 * Ns; idx += NT) {
                const int fl = idx / Ns, o = idx % Ns;
                const cx<T>* R = D[fl].R;
                cx<T> z[kLongBonds];
#pragma unroll
                for (int j = 0; j < kLongBonds; ++j) z[j] = cx<T>{T(0), T(0)};
                int f = 0;
                for (; f + 4 <= N; f += 4) {
                    cx<T> r[4];
#pragma unroll
                    for (int q = 0; q < 4; ++q) r[q] = R[size_t(f + q) * Ns + o];
#pragma unroll
                    for (int q = 0; q < 4; ++q)
#pragma unroll
                        for (int j = 0; j < kLongBonds; ++j)
                            if (j < nb) cmac(z[j], r[q], s_Cb[(j * 2 + fl) * Nmax + f + q]);
                }
                for (; f < N; ++f) {
                    const cx<T> r = R[size_t(f) * Ns + o];
#pragma unroll
                    for (int j = 0; j < kLongBonds; ++j)
                        if (j < nb) cmac(z[j], r, s_Cb[(j * 2 + fl) * Nmax + f]);
                }
#pragma unroll
                for (int j = 0; j < kLongBonds; ++j)
                    if (j < nb) s_Zb[j * 2 * Ns + idx] = z[j];
            }
            __syncthreads();
            for (int j = 0; j < nb; ++j) {
                const int code = s_bl[b0 + j], s0 = code & 0xFFFF, t0 = code >> 16;
                cx<T> m11[2];
                long_stage<T, NT>(J, w, s0, t0, s_fock, s_worb, s_coef, s_rowc, s_del, s_C, nullptr, s_pt, s_dd, s_red,
                                  m11);
                D[0].M11 = m11[0];
                D[1].M11 = m11[1];
                D[0].Z = s_Zb + j * 2 * Ns;
                D[1].Z = s_Zb + j * 2 * Ns + Ns;
                for (int k = tid; k < Nexc; k += NT) {
                    const cx<double> q = to_d(long_state_ratio<T>(D, cur, k, s_exu, s_exd, s_pre, Ns, nullptr));
                    s_S[k].x += q.x;
                    s_S[k].y += q.y;
                }
                __syncthreads();   // the next bond restages
            }
        }
        const double npar = double(2 * Ns - nanti), na = double(nanti);
        for (int k = tid; k < Nexc; k += NT) {
            int V[2], F[2], odd = 0;
            for (int fl = 0; fl < 2; ++fl) {
                const int n = long_hops(cur, k, fl, s_exu, s_exd, Ns, V, F);
                odd ^= long_hop_parity(s_pre + fl * (Ns + 1), n, V, F);
            }
            const double hs = odd ? -1.0 : 1.0;
            const cx<double> a = s_a[k], S = s_S[k];
            s_hh[k] = cx<double>{hs * (a.x * 0.25 * (npar - na) - 0.5 * S.x), hs * (a.y * 0.25 * (npar - na) - 0.5 * S.y)};
            s_a[k] = cx<double>{hs * a.x, hs * a.y};
        }
        __syncthreads();
        const double iw = 1.0 / wsum;
        cx<double>* H = J.pjx + size_t(w) * 2 * Nexc * Nexc;
        cx<double>* O = H + size_t(Nexc) * Nexc;
        // Mixed form: the outer products in FP32, summed over a block of
        // measurements and widened into the FP64 sums (ho_push, as the
        // transverse channel's measurement; FP64 products at once for a walker
        // whose factors exceed 1e15)
        bool narrow = false;
        if constexpr (sizeof(T) == 4) {
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
        if (lane == 0) s_red[warp] = double(m);
        __syncthreads();
        if (tid == 0) {
            double t = 0.0;
            for (int q = 0; q < NW; ++q) t += s_red[q];
            J.sm[w].x += t / double(Ns);
            J.sm_n[w] += 1;
        }
    }
}

// SlaterDeterminant::VirtUpdate (SlaterDeterminant.cpp:96-268) for hop sets of
// walker w in the longitudinal channel: hops[4 i .. 4 i + 3] = (up_from, up_to,
// dn_from, dn_to) is an exchange (up_to = dn_from, dn_to = up_from) or empty
// (-1); out[2 (k nset + i)] = q_k / Amp including the wavefunction's hop sign.
template <typename T, int NT>
__global__ void __launch_bounds__(NT) k_virt_long(DevJob J, int w, int nset, const int32_t* hops, double* out)
{
    extern __shared__ __align__(16) char smem[];
    if (blockIdx.x != 0 || w >= J.W) return;
    const int Ns = J.Ns, Nmax = J.Nmax, Nexc = J.Nexc, tid = threadIdx.x;
    const LongMeasLayout lay = long_meas_layout<T, NT>(Ns, Nmax, Nexc);
    long_load<T, NT>(J, w, lay, smem);
    const int16_t* s_fock = reinterpret_cast<const int16_t*>(smem + lay.fock);
    const int16_t* s_wslot = reinterpret_cast<const int16_t*>(smem + lay.wslot);
    const int16_t* s_worb = reinterpret_cast<const int16_t*>(smem + lay.worb);
    const int16_t* s_exu = reinterpret_cast<const int16_t*>(smem + lay.exu);
    const int16_t* s_exd = reinterpret_cast<const int16_t*>(smem + lay.exd);
    const int16_t* s_pre = reinterpret_cast<const int16_t*>(smem + lay.pre);
    const cx<T>* s_coef = reinterpret_cast<const cx<T>*>(smem + lay.coef);
    cx<T>* s_rowc = reinterpret_cast<cx<T>*>(smem + lay.rowc);
    cx<T>* s_del = reinterpret_cast<cx<T>*>(smem + lay.del);
    cx<T>* s_C = reinterpret_cast<cx<T>*>(smem + lay.C);
    cx<T>* s_Z = reinterpret_cast<cx<T>*>(smem + lay.Z);
    cx<T>* s_pt = reinterpret_cast<cx<T>*>(smem + lay.pt);
    cx<T>* s_dd = reinterpret_cast<cx<T>*>(smem + lay.dd);
    double* s_red = reinterpret_cast<double*>(smem + lay.red);
    const int cur = J.cur[w];
    LongFl<T> D[2];
    for (int fl = 0; fl < 2; ++fl) {
        D[fl].rowc = s_rowc + fl * Nmax;
        D[fl].del = s_del + fl * Nmax;
        D[fl].Z = s_Z + fl * Ns;
        D[fl].pt = s_pt + fl * Ns;
        D[fl].dd = s_dd + fl * Ns;
        D[fl].R = static_cast<const cx<T>*>(J.gup) + (size_t(w) * 2 + fl) * size_t(Nmax) * Ns;
        D[fl].wslot = s_wslot + fl * Ns;
        D[fl].Ns = Ns;
    }
    for (int i = 0; i < nset; ++i) {
        const int s0 = hops[4 * i], t0 = hops[4 * i + 1];
        const bool move = s0 >= 0;
        D[0].moved = D[1].moved = move;
        if (move) {
            cx<T> m11[2];
            long_stage<T, NT>(J, w, s0, t0, s_fock, s_worb, s_coef, s_rowc, s_del, s_C, s_Z, s_pt, s_dd, s_red, m11);
            D[0].M11 = m11[0];
            D[1].M11 = m11[1];
        }
        for (int k = tid; k < Nexc; k += NT) {
            int odd = 0;
            const cx<double> q = to_d(long_state_ratio<T>(D, cur, k, s_exu, s_exd, s_pre, Ns, &odd));
            const double hs = odd ? -1.0 : 1.0;
            out[2 * (size_t(k) * nset + i)] = hs * q.x;
            out[2 * (size_t(k) * nset + i) + 1] = hs * q.y;
        }
        __syncthreads();
    }
}

}  // namespace
}  // namespace gv
