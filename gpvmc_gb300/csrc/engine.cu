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
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "device.cuh"
#include "kernels.cuh"
#include "kernels_trans.cuh"
#include "kernels_long.cuh"
#include "kernels_res.cuh"
#include "kernels_tc.cuh"
#include "kernels_trans_res.cuh"
#include "model.hpp"

using namespace gv;

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
    // tensor-core StatSpinStruct: the antiparallel counts run on a second
    // stream beside the pair kernel (forked from and joined back into stream)
    cudaStream_t side = nullptr;
    cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
    DevJob d{};
    std::vector<void*> allocs;
    bool ready = false;
    int nt = 128;
    double last_ms = 0.0;
    int64_t last_launches = 0;
    int64_t total_launches = 0;
    int64_t timer_launch0 = 0;
    cudaEvent_t tev0 = nullptr, tev1 = nullptr;
    // per-launch event pairs while the timer runs: kind 0 walk, 1 re-inversion, 2 measurement
    bool timing = false;
    std::vector<cudaEvent_t> ev_pool;
    std::vector<std::pair<int, int>> ev_used;   // (kind, index of first event of the pair)
    double kind_ms[3] = {0, 0, 0};
    int64_t kind_n[3] = {0, 0, 0};
    std::vector<double> kind_each[3];
    std::vector<double> wphi, wneel;
    std::vector<uint64_t> start_draws;   // Philox stream-1 uniform index per walker
    int n_sm = 1;                        // SMs of the job's device (persistent grids)
    bool trans = false;                  // transverse-exciton channel
    bool lng = false;                    // longitudinal-exciton channel
    struct WalkGraph {
        cudaGraphExec_t exec;
        int64_t launches;
    };
    std::map<std::tuple<uint64_t, uint64_t, int, bool>, WalkGraph> graphs;   // GV_FLAG_CUDA_GRAPHS
    bool graphs_off = false;
    int64_t graph_replays = 0;
    std::vector<int16_t> exu, exd;       // channel tables (Channel::exc_up / exc_dn)
    // single-walker stepping: the proposal gv_job_trystep evaluated, waiting for gv_job_step
    struct Pending {
        int w = -1, v1 = 0, v2 = 0, khop = -1;
    } pend;
    gv_trace* step_trace = nullptr;      // device record of a single-walker step
    void* diag = nullptr;                // scratch of the diagnostic entry points (grown on demand)
    size_t diag_bytes = 0;
};

namespace {

thread_local const char* g_last_cuda_error = "";

// Bytes this library copied host -> device and device -> host (every copy
// goes through copy_async / copy_sync), for end-to-end accounting.
std::atomic<uint64_t> g_bytes_h2d{0}, g_bytes_d2h{0};

void count_copy(size_t n, cudaMemcpyKind k)
{
    if (k == cudaMemcpyHostToDevice) g_bytes_h2d += n;
    else if (k == cudaMemcpyDeviceToHost) g_bytes_d2h += n;
}

cudaError_t copy_async(void* dst, const void* src, size_t n, cudaMemcpyKind k, cudaStream_t s)
{
    count_copy(n, k);
    return cudaMemcpyAsync(dst, src, n, k, s);
}

cudaError_t copy_sync(void* dst, const void* src, size_t n, cudaMemcpyKind k)
{
    count_copy(n, k);
    return cudaMemcpy(dst, src, n, k);
}

// Status for a failed CUDA call, remembering its message for gv_last_cuda_error.
gv_status cuda_status(cudaError_t e)
{
    if (e == cudaSuccess) return GV_OK;
    g_last_cuda_error = cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? GV_ERR_OOM : GV_ERR_CUDA;
}

#define GV_CK(x)                                                   \
    do {                                                           \
        cudaError_t e_ = (x);                                      \
        if (e_ != cudaSuccess) return cuda_status(e_);             \
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

// Device scratch for the diagnostic entry points (VirtUpdate, drift, traces,
// start-state overlaps): allocated once and grown when a call needs more, so
// that repeated calls allocate nothing.  Every user finishes (synchronises)
// before it returns, so one buffer per job serves them all.
gv_status diag_scratch(gv_job* j, size_t bytes, void** out)
{
    bytes = (bytes + 255) & ~size_t(255);
    if (bytes > j->diag_bytes) {
        if (j->diag) {
            GV_CK(cudaStreamSynchronize(j->stream));
            cudaFree(j->diag);
            j->diag = nullptr;
            j->diag_bytes = 0;
        }
        GV_CK(cudaMalloc(&j->diag, bytes));
        j->diag_bytes = bytes;
    }
    *out = j->diag;
    return GV_OK;
}

// Two regions of one diagnostic scratch: a at offset 0, b at the next 256-byte boundary.
template <typename A, typename B>
gv_status diag_pair(gv_job* j, size_t na, size_t nb, A** a, B** b)
{
    const size_t off = (sizeof(A) * na + 255) & ~size_t(255);
    void* p = nullptr;
    gv_status st = diag_scratch(j, off + sizeof(B) * nb, &p);
    if (st) return st;
    *a = static_cast<A*>(p);
    *b = reinterpret_cast<B*>(static_cast<char*>(p) + off);
    return GV_OK;
}

bool valid_config(const gv_job_config* c)
{
    if (!c) return false;
    if (c->L < 4 || c->L > 64 || (c->L % 2)) return false;
    if (c->channel == GV_CH_TRANS && c->L > 32) return false;
    if (c->channel == GV_CH_LONG && c->L > 24) return false;   // its walk stages 3 x 2 x L^2 orbitals on chip
    if (c->channel != GV_CH_GROUNDSTATE && c->channel != GV_CH_TRANS && c->channel != GV_CH_LONG) return false;
    if (c->channel != GV_CH_GROUNDSTATE && (c->flags & GV_FLAG_DELAYED_UPDATES)) return false;
    if (c->n_walkers < 1 || c->n_walkers > (1 << 20)) return false;
    if (c->precision != GV_PREC_FP64 && c->precision != GV_PREC_MIXED) return false;
    if (c->reinv_every < 0) return false;
    if (c->flags & ~(GV_FLAG_REINV_DEFERRED | GV_FLAG_REINV_ON_DRIFT | GV_FLAG_DELAYED_UPDATES | GV_FLAG_STREAM_INVERSES |
                     GV_FLAG_SCALAR_PAIRS | GV_FLAG_CUDA_GRAPHS | GV_FLAG_TC_PROJHEIS))
        return false;
    // ProjHeis from the tensor-core pair products: mixed ground state, N <= 128
    if ((c->flags & GV_FLAG_TC_PROJHEIS) &&
        (c->channel != GV_CH_GROUNDSTATE || c->precision != GV_PREC_MIXED || c->L * c->L / 2 > kTcM ||
         (c->flags & GV_FLAG_SCALAR_PAIRS)))
        return false;
    if ((c->flags & GV_FLAG_REINV_ON_DRIFT) && (!(c->flags & GV_FLAG_REINV_DEFERRED) || !(c->drift_threshold > 0.0)))
        return false;
    return true;
}

int pick_threads(int Nmax) { return Nmax > 128 ? 256 : 128; }

// Either exciton channel: a wavefunction with several states, its Fock state,
// sign, current state and weight kept per walker.
inline bool exc(const gv_job* j) { return j->trans || j->lng; }

// Exciton channel tables, checked against the channel's hop table
// (WaveFunction::m_exc, WaveFunction.cpp:39-67): from state a, state b != a
// must be the flavour-0 hop exc_up[a] -> exc_up[b] and the flavour-1 hop
// exc_dn[b] -> exc_dn[a], the structure the exciton kernels rely on.
bool trans_tables(const Channel& ch, std::vector<int16_t>& up, std::vector<int16_t>& dn)
{
    const int n = ch.Nexc;
    if (n < 2 || int(ch.exc_up.size()) != n || int(ch.exc_dn.size()) != n) return false;
    up.assign(n, 0);
    dn.assign(n, 0);
    for (int k = 0; k < n; ++k) { up[k] = int16_t(ch.exc_up[k]); dn[k] = int16_t(ch.exc_dn[k]); }
    for (int a = 0; a < n; ++a)
        for (int b = 0; b < n; ++b) {
            const size_t i = (size_t(a) * n + b) * 2;
            if (a == b) {
                if (ch.hop_from[i] >= 0 || ch.hop_from[i + 1] >= 0) return false;
                continue;
            }
            if (ch.hop_from[i] != up[a] || ch.hop_to[i] != up[b] || ch.hop_from[i + 1] != dn[b] ||
                ch.hop_to[i + 1] != dn[a])
                return false;
        }
    return true;
}

// The wavefunction's Fock state on the host (State, State.cpp): slot of every
// orbital (-1 empty), orbital of every slot, sign, channel state.
struct WavHost {
    std::vector<int16_t> slot[2], orb[2];
    int sign = 1, cur = 0;
};

WavHost wav_state0(const gv_job* j)
{
    WavHost s;
    for (int fl = 0; fl < 2; ++fl) {
        s.slot[fl].assign(j->Ns, -1);
        s.orb[fl].assign(j->Nmax, 0);
        for (int x = 0; x < j->Ns; ++x)
            if (j->ch.fock0[fl][x] < j->ch.N[fl]) {
                s.slot[fl][x] = int16_t(j->ch.fock0[fl][x]);
                s.orb[fl][j->ch.fock0[fl][x]] = int16_t(x);
            }
    }
    return s;
}

// WaveFunction::Hop to state k (WaveFunction.cpp:69-73): State::Hop with the
// sign of State::HopSign (State.cpp:73-115), parities taken before the hop.
void wav_hop(const gv_job* j, WavHost& s, int k)
{
    const Channel& ch = j->ch;
    const size_t i = (size_t(s.cur) * ch.Nexc + k) * 2;
    int odd = 0;
    for (int fl = 0; fl < 2; ++fl) {
        const int from = ch.hop_from[i + fl], to = ch.hop_to[i + fl];
        if (from < 0) continue;
        for (int x = std::min(from, to) + 1; x < std::max(from, to); ++x) odd ^= s.slot[fl][x] >= 0 ? 1 : 0;
    }
    s.sign *= odd ? -1 : 1;
    for (int fl = 0; fl < 2; ++fl) {
        const int from = ch.hop_from[i + fl], to = ch.hop_to[i + fl];
        if (from < 0) continue;
        const int16_t p = s.slot[fl][from];
        s.slot[fl][from] = -1;
        s.slot[fl][to] = p;
        s.orb[fl][p] = int16_t(to);
    }
    s.cur = k;
}

// WaveFunction::Hop in the longitudinal channel: up to two hops per flavour
// (State::get_hop_path pairs, State::HopSign with the second hop counted after
// the first, State.cpp:73-115).
void long_wav_hop(const gv_job* j, WavHost& s, int k)
{
    int odd = 0;
    for (int fl = 0; fl < 2; ++fl) {
        int V[2], F[2];
        const int n = long_hops(s.cur, k, fl, j->exu.data(), j->exd.data(), j->Ns, V, F);
        std::vector<int16_t> sl = s.slot[fl];
        for (int i = 0; i < n; ++i) {
            for (int x = std::min(V[i], F[i]) + 1; x < std::max(V[i], F[i]); ++x) odd ^= sl[x] >= 0 ? 1 : 0;
            const int16_t r = sl[V[i]];
            sl[V[i]] = -1;
            sl[F[i]] = r;
        }
        for (int i = 0; i < n; ++i) {
            const int16_t r = s.slot[fl][V[i]];
            s.slot[fl][V[i]] = -1;
            s.slot[fl][F[i]] = r;
            s.orb[fl][r] = int16_t(F[i]);
        }
    }
    s.sign *= odd ? -1 : 1;
    s.cur = k;
}

size_t scratch_walkers(const gv_job* j) { return size_t(j->W); }

// Raise (never lower) a kernel's dynamic shared-memory limit on the current
// device.  Jobs driven from different host threads launch the same kernel
// instantiation with different sizes; a per-launch cudaFuncSetAttribute
// could lower the limit between another thread's set and its launch.
cudaError_t raise_smem_limit(const void* fn, size_t bytes)
{
    static std::mutex mu;
    static std::map<std::pair<int, const void*>, size_t> limit;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lk(mu);
    size_t& cur = limit[{dev, fn}];
    if (bytes <= cur) return cudaSuccess;
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(bytes));
    if (e == cudaSuccess) cur = bytes;
    return e;
}

template <typename K>
cudaError_t raise_smem_limit(K* kernel, size_t bytes)
{
    return raise_smem_limit(reinterpret_cast<const void*>(kernel), bytes);
}

cudaError_t mark_begin(gv_job* j, int kind, int* slot)
{
    *slot = -1;
    if (!j->timing) return cudaSuccess;
    const size_t need = 2 * (j->ev_used.size() + 1);
    while (j->ev_pool.size() < need) {
        cudaEvent_t e;
        cudaError_t r = cudaEventCreate(&e);
        if (r) return r;
        j->ev_pool.push_back(e);
    }
    *slot = int(2 * j->ev_used.size());
    j->ev_used.push_back({kind, *slot});
    return cudaEventRecord(j->ev_pool[*slot], j->stream);
}

cudaError_t mark_end(gv_job* j, int slot)
{
    if (slot < 0) return cudaSuccess;
    return cudaEventRecord(j->ev_pool[slot + 1], j->stream);
}

template <typename T, int NT, int KD>
gv_status launch_walk(gv_job* j, uint64_t nsteps, uint64_t s0, uint64_t meas, int mask, int measure_first)
{
    const bool inkernel = !(j->cfg.flags & GV_FLAG_REINV_DEFERRED);
    const WalkLayout lay = walk_layout<T, NT, KD>(j->Ns, j->Nmax, (mask & GV_MEAS_PROJHEIS) != 0, inkernel);
    GV_CK(raise_smem_limit(k_walk_gs<T, NT, KD>, lay.total));
    // shared-memory carveout for up to 8 resident walkers per SM, the rest stays L1
    const int carve = int(std::min<size_t>(100, (8 * (lay.total + 1024) * 100 + 233471) / 233472));
    GV_CK(cudaFuncSetAttribute(k_walk_gs<T, NT, KD>, cudaFuncAttributePreferredSharedMemoryCarveout, carve));
    int slot;
    GV_CK(mark_begin(j, 0, &slot));
    k_walk_gs<T, NT, KD><<<j->W, NT, lay.total, j->stream>>>(j->d, nsteps, s0, meas, mask, inkernel ? 1 : 0,
                                                              measure_first);
    GV_CK(cudaGetLastError());
    GV_CK(mark_end(j, slot));
    ++j->last_launches;
    ++j->total_launches;
    return GV_OK;
}

#ifndef GV_DELAY_DEPTH
#define GV_DELAY_DEPTH 4
#endif
constexpr int kDelay = GV_DELAY_DEPTH;

// On-chip walk (both FP32 inverses in TMEM / shared memory for the whole call):
// mixed ground state, N <= 128 and even (rows of the inverses and of the phase
// table are copied in 16-byte pieces), deferred re-inversion, no delayed updates.
bool resident_ok(const gv_job* j, uint64_t nsteps)
{
    const int f = j->cfg.flags;
    return nsteps > 0 && !exc(j) && j->cfg.precision == GV_PREC_MIXED && j->N[0] == j->N[1] && j->Nmax <= 128 &&
           j->Nmax % 2 == 0 && j->Nk % 2 == 0 && (f & GV_FLAG_REINV_DEFERRED) && !(f & GV_FLAG_DELAYED_UPDATES) &&
           !(f & GV_FLAG_STREAM_INVERSES);
}

gv_status launch_walk_res(gv_job* j, uint64_t nsteps, uint64_t s0, uint64_t meas, int mask)
{
    const ResLayout lay = res_layout(j->Ns, j->N[0], (mask & GV_MEAS_PROJHEIS) != 0);
    GV_CK(raise_smem_limit(k_walk_gs_res, lay.total));
    GV_CK(cudaFuncSetAttribute(k_walk_gs_res, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
    int slot;
    GV_CK(mark_begin(j, 0, &slot));
    k_walk_gs_res<<<j->W, kResThreads, lay.total, j->stream>>>(j->d, nsteps, s0, meas, mask);
    GV_CK(cudaGetLastError());
    GV_CK(mark_end(j, slot));
    ++j->last_launches;
    ++j->total_launches;
    return GV_OK;
}

// Delayed updates (depth kDelay) when requested and every particle column has its
// own thread; otherwise immediate rank-1 updates.
gv_status walk_dispatch(gv_job* j, uint64_t nsteps, uint64_t s0, uint64_t meas, int mask, int measure_first = 0)
{
    if (!measure_first && resident_ok(j, nsteps)) return launch_walk_res(j, nsteps, s0, meas, mask);
    const bool fp64 = j->cfg.precision == GV_PREC_FP64;
    const bool delayed = (j->cfg.flags & GV_FLAG_DELAYED_UPDATES) && j->Nmax <= j->nt;
    if (j->nt == 128) {
        if (delayed) return fp64 ? launch_walk<double, 128, kDelay>(j, nsteps, s0, meas, mask, measure_first)
                                 : launch_walk<float, 128, kDelay>(j, nsteps, s0, meas, mask, measure_first);
        return fp64 ? launch_walk<double, 128, 0>(j, nsteps, s0, meas, mask, measure_first)
                    : launch_walk<float, 128, 0>(j, nsteps, s0, meas, mask, measure_first);
    }
    if (delayed) return fp64 ? launch_walk<double, 256, kDelay>(j, nsteps, s0, meas, mask, measure_first)
                             : launch_walk<float, 256, kDelay>(j, nsteps, s0, meas, mask, measure_first);
    return fp64 ? launch_walk<double, 256, 0>(j, nsteps, s0, meas, mask, measure_first)
                : launch_walk<float, 256, 0>(j, nsteps, s0, meas, mask, measure_first);
}

template <typename T, int NT>
gv_status launch_check(gv_job* j, double threshold)
{
    size_t sm = check_smem_bytes(j->Nmax, NT) + 64;
    // Gauss-Jordan matrix in shared memory: always while two CTAs still fit per
    // SM, and for the outright cadence (every due walker re-inverted) while it fits at all
    const size_t msz = sizeof(cx<double>) * size_t(j->Nmax) * j->Nmax;
    const int m_in_smem = (sm + msz <= size_t(113) * 1024 || (threshold < 0.0 && sm + msz <= size_t(200) * 1024)) ? 1 : 0;
    if (m_in_smem) sm += msz;
    GV_CK(raise_smem_limit(k_check_reinvert<T, NT>, sm));
    int slot;
    GV_CK(mark_begin(j, 1, &slot));
    k_check_reinvert<T, NT><<<j->W, NT, sm, j->stream>>>(j->d, threshold, m_in_smem);
    GV_CK(cudaGetLastError());
    GV_CK(mark_end(j, slot));
    ++j->last_launches;
    ++j->total_launches;
    return GV_OK;
}

// Deferred cadence: walkers past reinv_every accepted exchanges are checked
// (GV_FLAG_REINV_ON_DRIFT) or re-inverted outright.
gv_status deferred_reinversion(gv_job* j)
{
    const double thr = (j->cfg.flags & GV_FLAG_REINV_ON_DRIFT) ? j->cfg.drift_threshold : -1.0;
    return j->cfg.precision == GV_PREC_FP64 ? launch_check<double, 256>(j, thr) : launch_check<float, 256>(j, thr);
}

constexpr int kTrackMask = GV_MEAS_STAGMAGN_TRACK | GV_MEAS_OVERLAP_TRACK;
constexpr int kInnerMask = GV_MEAS_PROJHEIS | GV_MEAS_STAGMAGN;   // measured inside the walk / measure kernels

gv_status tracks_dispatch(gv_job* j, int mask)
{
    if (!j->d.track_cap) return GV_OK;
    int slot;
    GV_CK(mark_begin(j, 2, &slot));
    k_tracks<<<(j->W + 7) / 8, 256, 0, j->stream>>>(j->d, mask);
    GV_CK(cudaGetLastError());
    GV_CK(mark_end(j, slot));
    ++j->last_launches;
    ++j->total_launches;
    return GV_OK;
}

// Tensor-core exciton overlap rows Z = GupT^T Phi_0: mixed exciton channel with
// Nexc <= 128, N1 <= 128, N0 <= 160.
bool trans_z_tc_ok(const gv_job* j)
{
    return j->trans && j->cfg.precision == GV_PREC_MIXED && j->ch.Nexc <= kTcM && j->N[1] <= kTcM &&
           j->N[0] <= kTcMaxK && !(j->cfg.flags & GV_FLAG_SCALAR_PAIRS);
}

// Tensor-core overlap sums of the longitudinal measurement: mixed, N <= 128,
// the Z buffer (W x 2 flavours x 2 Ns bonds x Ns/2 upper-band orbitals,
// complex FP32) at most 8 GB.
bool long_z_tc_ok(const gv_job* j)
{
    return j->lng && j->cfg.precision == GV_PREC_MIXED && j->N[0] == j->N[1] && j->N[0] <= kTcM &&
           j->Ns <= kOccMaxNs && size_t(j->W) * 2 * j->Ns * j->Ns * sizeof(cx<float>) <= (size_t(8) << 30) &&
           !(j->cfg.flags & GV_FLAG_SCALAR_PAIRS);
}

// Tensor-core StatSpinStruct: mixed ground state with N_0 = N_1 <= 128.
bool statspin_tc_ok(const gv_job* j)
{
    return !exc(j) && j->cfg.precision == GV_PREC_MIXED && j->N[0] == j->N[1] && j->N[0] <= kTcM &&
           j->Ns <= kTcThreads && j->Ns <= kOccMaxNs && !(j->cfg.flags & GV_FLAG_SCALAR_PAIRS);
}

// mode bit 0: StatSpinStruct; bit 1: ProjHeis from the tensor-core pair products
// (GV_FLAG_TC_PROJHEIS).
gv_status statspin_dispatch(gv_job* j, int mode = 1)
{
    if (statspin_tc_ok(j)) {
        const TcLayout lay = tc_layout(j->N[0]);
        GV_CK(raise_smem_limit(k_statspin_tc, lay.total));
        int slot;
        GV_CK(mark_begin(j, 2, &slot));
        const bool side = (mode & 1) && j->side;
        if (mode & 1) {   // antiparallel counts from occupation bitsets (Aud: no overlap with the pair sums)
            cudaStream_t s = j->stream;
            if (side) {   // beside the pair kernel, which holds one CTA per SM
                GV_CK(cudaEventRecord(j->fork_ev, j->stream));
                GV_CK(cudaStreamWaitEvent(j->side, j->fork_ev, 0));
                s = j->side;
            }
            k_occ_bits<<<(j->W + 31) / 32, 256, 0, s>>>(j->d, j->d.occ);
            k_occ_pairs<<<j->Ns, 256, 0, s>>>(j->d, j->d.occ);
            GV_CK(cudaGetLastError());
            if (side) GV_CK(cudaEventRecord(j->join_ev, j->side));
            j->last_launches += 2;
            j->total_launches += 2;
        }
        k_statspin_tc<<<std::min(j->W, j->n_sm), kTcBlock, lay.total, j->stream>>>(j->d, mode);
        GV_CK(cudaGetLastError());
        if (side) GV_CK(cudaStreamWaitEvent(j->stream, j->join_ev, 0));   // joined before anything reads the sums
        if (mode & 1) {
            k_fold_ss<<<j->n_sm, 256, 0, j->stream>>>(j->d);
            GV_CK(cudaGetLastError());
            ++j->last_launches;
            ++j->total_launches;
        }
        GV_CK(mark_end(j, slot));
        ++j->last_launches;
        ++j->total_launches;
        return GV_OK;
    }
    const bool fp64 = j->cfg.precision == GV_PREC_FP64;
    size_t sm = (fp64 ? sizeof(cx<double>) : sizeof(cx<float>)) * 4 * j->Nmax + sizeof(int16_t) * 2 * j->Nmax + 16;
    int slot;
    GV_CK(mark_begin(j, 2, &slot));
    if (fp64) k_statspin<double, 128><<<j->W, 128, sm, j->stream>>>(j->d);
    else k_statspin<float, 128><<<j->W, 128, sm, j->stream>>>(j->d);
    GV_CK(cudaGetLastError());
    GV_CK(mark_end(j, slot));
    ++j->last_launches;
    ++j->total_launches;
    return GV_OK;
}

template <typename T, int NT>
gv_status launch_invert(gv_job* j, int only_due)
{
    size_t sm = gj_smem_bytes(j->Nmax, NT) + 64;
    const size_t msz = sizeof(cx<double>) * size_t(j->Nmax) * j->Nmax;
    const int m_in_smem = (sm + msz <= size_t(200) * 1024) ? 1 : 0;   // N <= 112
    if (m_in_smem) sm += msz;
    GV_CK(raise_smem_limit(k_invert<T, NT>, sm));
    int slot;
    GV_CK(mark_begin(j, 1, &slot));
    k_invert<T, NT><<<j->W, NT, sm, j->stream>>>(j->d, only_due, m_in_smem);
    GV_CK(cudaGetLastError());
    GV_CK(mark_end(j, slot));
    ++j->total_launches;
    return GV_OK;
}

gv_status invert_all(gv_job* j, int only_due = 0)
{
    return j->cfg.precision == GV_PREC_FP64 ? launch_invert<double, 256>(j, only_due)
                                            : launch_invert<float, 256>(j, only_due);
}

template <typename T>
gv_status launch_walk_trans(gv_job* j, uint64_t nsteps)
{
    constexpr int NT = 256;
    const bool inkernel = !(j->cfg.flags & GV_FLAG_REINV_DEFERRED);
    const TransLayout lay = trans_layout<T, NT>(j->Ns, j->Nmax, j->ch.Nexc, inkernel);
    GV_CK(raise_smem_limit(k_walk_trans<T, NT>, lay.total));
    int slot;
    GV_CK(mark_begin(j, 0, &slot));
    k_walk_trans<T, NT><<<j->W, NT, lay.total, j->stream>>>(j->d, nsteps, inkernel ? 1 : 0);
    GV_CK(cudaGetLastError());
    GV_CK(mark_end(j, slot));
    ++j->last_launches;
    ++j->total_launches;
    return GV_OK;
}

// On-chip exciton walk (GupT and the flavour-1 inverse in TMEM, the flavour-0
// inverse in shared memory): mixed, Nexc <= 128, deferred re-inversion.
constexpr size_t kMaxSmemPerBlock = 227 * 1024;   // opt-in dynamic shared memory per block on sm_100 / sm_103

bool trans_resident_ok(const gv_job* j, uint64_t nsteps)
{
    const int f = j->cfg.flags;
    // the staged phase rows are copied whole (8 Nk bytes: a multiple of 16)
    return nsteps > 0 && j->trans && j->cfg.precision == GV_PREC_MIXED &&
           trans_res_fits(j->N[0], j->N[1], j->ch.Nexc) && j->Nk % 2 == 0 &&
           trans_res_layout(j->Ns, j->Nk, j->Nmax, j->N[0], j->ch.Nexc).total <= kMaxSmemPerBlock &&
           (f & GV_FLAG_REINV_DEFERRED) && !(f & GV_FLAG_STREAM_INVERSES);
}

gv_status launch_walk_trans_res(gv_job* j, uint64_t nsteps)
{
    const TrResLayout lay = trans_res_layout(j->Ns, j->Nk, j->Nmax, j->N[0], j->ch.Nexc);
    GV_CK(raise_smem_limit(k_walk_trans_res, lay.total));
    GV_CK(cudaFuncSetAttribute(k_walk_trans_res, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
    int slot;
    GV_CK(mark_begin(j, 0, &slot));
    k_walk_trans_res<<<j->W, kTrThreads, lay.total, j->stream>>>(j->d, nsteps);
    GV_CK(cudaGetLastError());
    GV_CK(mark_end(j, slot));
    ++j->last_launches;
    ++j->total_launches;
    return GV_OK;
}

gv_status walk_trans_dispatch(gv_job* j, uint64_t nsteps)
{
    if (trans_resident_ok(j, nsteps)) return launch_walk_trans_res(j, nsteps);
    return j->cfg.precision == GV_PREC_FP64 ? launch_walk_trans<double>(j, nsteps) : launch_walk_trans<float>(j, nsteps);
}

template <typename T>
gv_status launch_measure_trans(gv_job* j, int mask)
{
    constexpr int NT = 256;
    const MeasLayout lay = meas_layout<T, NT>(j->Ns, j->Nmax, j->ch.Nexc);
    const cx<float>* zpre = nullptr;
    if (j->d.zbuf && (mask & GV_MEAS_PROJHEIS)) {   // Z = GupT^T Phi_0 on the tensor cores first
        const TcLayout zl = tc_layout_z(j->N[1]);
        GV_CK(raise_smem_limit(k_trans_z_tc, zl.total));
        int zs;
        GV_CK(mark_begin(j, 2, &zs));
        k_trans_z_tc<<<std::min(j->W, j->n_sm), kTcBlock, zl.total, j->stream>>>(j->d, j->d.zbuf);
        GV_CK(cudaGetLastError());
        GV_CK(mark_end(j, zs));
        ++j->last_launches;
        ++j->total_launches;
        zpre = j->d.zbuf;
    }
    GV_CK(raise_smem_limit(k_measure_trans<T, NT>, lay.total));
    int slot;
    GV_CK(mark_begin(j, 2, &slot));
    k_measure_trans<T, NT><<<j->W, NT, lay.total, j->stream>>>(j->d, mask, zpre);
    GV_CK(cudaGetLastError());
    GV_CK(mark_end(j, slot));
    ++j->last_launches;
    ++j->total_launches;
    return GV_OK;
}

gv_status measure_trans_dispatch(gv_job* j, int mask)
{
    return j->cfg.precision == GV_PREC_FP64 ? launch_measure_trans<double>(j, mask) : launch_measure_trans<float>(j, mask);
}

// sigma (and, with out, every state's |rho0_k|^2) of every walker.
// Longitudinal exciton: the walk, the ProjHeis / StagMagnZ measurement, the
// state overlaps (start-state pick, weight) and VirtUpdate.
template <typename T>
gv_status launch_walk_long(gv_job* j, uint64_t nsteps)
{
    constexpr int NT = 256;
    const bool inkernel = !(j->cfg.flags & GV_FLAG_REINV_DEFERRED);
    const LongLayout lay = long_layout<T, NT>(j->Ns, j->Nmax, j->ch.Nexc, inkernel);
    GV_CK(raise_smem_limit(k_walk_long<T, NT>, lay.total));
    int slot;
    GV_CK(mark_begin(j, 0, &slot));
    k_walk_long<T, NT><<<j->W, NT, lay.total, j->stream>>>(j->d, nsteps, inkernel ? 1 : 0);
    GV_CK(cudaGetLastError());
    GV_CK(mark_end(j, slot));
    ++j->last_launches;
    ++j->total_launches;
    return GV_OK;
}

gv_status walk_long_dispatch(gv_job* j, uint64_t nsteps)
{
    return j->cfg.precision == GV_PREC_FP64 ? launch_walk_long<double>(j, nsteps) : launch_walk_long<float>(j, nsteps);
}

template <typename T>
gv_status launch_measure_long(gv_job* j, int mask)
{
    constexpr int NT = 256;
    const LongMeasLayout lay = long_meas_layout<T, NT>(j->Ns, j->Nmax, j->ch.Nexc);
    const cx<float>* zpre = nullptr;
    if (sizeof(T) == 4 && j->d.zbuf && (mask & GV_MEAS_PROJHEIS)) {   // the bonds' Z on the tensor cores first
        const TcLayout zl = tc_layout_lz(j->N[0]);
        GV_CK(raise_smem_limit(k_long_z_tc, zl.total));
        int zs;
        GV_CK(mark_begin(j, 2, &zs));
        k_long_z_tc<<<std::min(j->W, j->n_sm), kTcBlock, zl.total, j->stream>>>(j->d, j->d.zbuf);
        GV_CK(cudaGetLastError());
        GV_CK(mark_end(j, zs));
        ++j->last_launches;
        ++j->total_launches;
        zpre = j->d.zbuf;
    }
    GV_CK(raise_smem_limit(k_measure_long<T, NT>, lay.total));
    int slot;
    GV_CK(mark_begin(j, 2, &slot));
    k_measure_long<T, NT><<<j->W, NT, lay.total, j->stream>>>(j->d, mask, zpre);
    GV_CK(cudaGetLastError());
    GV_CK(mark_end(j, slot));
    ++j->last_launches;
    ++j->total_launches;
    return GV_OK;
}

gv_status measure_long_dispatch(gv_job* j, int mask)
{
    return j->cfg.precision == GV_PREC_FP64 ? launch_measure_long<double>(j, mask) : launch_measure_long<float>(j, mask);
}

gv_status long_states(gv_job* j, double* out)
{
    constexpr int NT = 256;
    const size_t sm = ((sizeof(int16_t) * (4 * size_t(j->Ns) + 2) + 15) & ~size_t(15)) + sizeof(double) * (NT / 32);
    if (j->cfg.precision == GV_PREC_FP64) k_long_states<double, NT><<<j->W, NT, sm, j->stream>>>(j->d, out);
    else k_long_states<float, NT><<<j->W, NT, sm, j->stream>>>(j->d, out);
    GV_CK(cudaGetLastError());
    ++j->total_launches;
    return GV_OK;
}

gv_status virt_update_long(gv_job* j, int walker, int nset, const int32_t* hops, double* out)
{
    for (int i = 0; i < nset; ++i) {
        const int32_t* h = hops + 4 * i;
        const bool empty = h[0] < 0 && h[1] < 0 && h[2] < 0 && h[3] < 0;
        for (int q = 0; q < 4; ++q)
            if (h[q] < -1 || h[q] >= j->Ns) return GV_ERR_INVALID;
        if (!empty && (h[0] < 0 || h[1] < 0 || h[2] != h[1] || h[3] != h[0])) return GV_ERR_INVALID;   // exchanges only
    }
    if (nset == 0) return GV_OK;
    {   // each exchange moves a flavour-0 particle from up_from and a flavour-1 particle from dn_from
        std::vector<int16_t> fock(2 * size_t(j->Ns));
        GV_CK(cudaStreamSynchronize(j->stream));
        GV_CK(copy_sync(fock.data(), j->d.fock + size_t(walker) * 2 * j->Ns, fock.size() * sizeof(int16_t),
                        cudaMemcpyDeviceToHost));
        for (int i = 0; i < nset; ++i)
            if (hops[4 * i] >= 0 && (fock[hops[4 * i]] < 0 || fock[j->Ns + hops[4 * i + 2]] < 0)) return GV_ERR_INVALID;
    }
    constexpr int NT = 256;
    int32_t* dh = nullptr;
    double* dout = nullptr;
    const size_t nout = size_t(2) * nset * j->ch.Nexc;
    gv_status st = diag_pair(j, size_t(4) * nset, nout, &dh, &dout);
    if (st) return st;
    cudaError_t e = copy_async(dh, hops, sizeof(int32_t) * 4 * nset, cudaMemcpyHostToDevice, j->stream);
    if (!e) {
        if (j->cfg.precision == GV_PREC_FP64) {
            const size_t sm = long_meas_layout<double, NT>(j->Ns, j->Nmax, j->ch.Nexc).total;
            e = raise_smem_limit(k_virt_long<double, NT>, sm);
            if (!e) k_virt_long<double, NT><<<1, NT, sm, j->stream>>>(j->d, walker, nset, dh, dout);
        } else {
            const size_t sm = long_meas_layout<float, NT>(j->Ns, j->Nmax, j->ch.Nexc).total;
            e = raise_smem_limit(k_virt_long<float, NT>, sm);
            if (!e) k_virt_long<float, NT><<<1, NT, sm, j->stream>>>(j->d, walker, nset, dh, dout);
        }
        if (!e) e = cudaGetLastError();
    }
    if (!e) e = copy_async(out, dout, sizeof(double) * nout, cudaMemcpyDeviceToHost, j->stream);
    if (!e) e = cudaStreamSynchronize(j->stream);
    return cuda_status(e);
}

gv_status trans_overlaps(gv_job* j, double* out)
{
    if (j->cfg.precision == GV_PREC_FP64) k_trans_overlaps<double, 128><<<j->W, 128, 0, j->stream>>>(j->d, out);
    else k_trans_overlaps<float, 128><<<j->W, 128, 0, j->stream>>>(j->d, out);
    GV_CK(cudaGetLastError());
    ++j->total_launches;
    return GV_OK;
}

gv_status upload_wav(gv_job* j, const std::vector<WavHost>& ws)
{
    const int W = j->W, Ns = j->Ns, Nmax = j->Nmax;
    std::vector<int16_t> slot(size_t(W) * 2 * Ns), orb(size_t(W) * 2 * Nmax);
    std::vector<int32_t> cur(W), sign(W);
    for (int w = 0; w < W; ++w) {
        for (int fl = 0; fl < 2; ++fl) {
            std::copy(ws[w].slot[fl].begin(), ws[w].slot[fl].end(), slot.begin() + (size_t(w) * 2 + fl) * Ns);
            std::copy(ws[w].orb[fl].begin(), ws[w].orb[fl].end(), orb.begin() + (size_t(w) * 2 + fl) * Nmax);
        }
        cur[w] = ws[w].cur;
        sign[w] = ws[w].sign;
    }
    GV_CK(copy_async(j->d.wslot, slot.data(), slot.size() * sizeof(int16_t), cudaMemcpyHostToDevice, j->stream));
    GV_CK(copy_async(j->d.worb, orb.data(), orb.size() * sizeof(int16_t), cudaMemcpyHostToDevice, j->stream));
    GV_CK(copy_async(j->d.cur, cur.data(), W * sizeof(int32_t), cudaMemcpyHostToDevice, j->stream));
    GV_CK(copy_async(j->d.wsign, sign.data(), W * sizeof(int32_t), cudaMemcpyHostToDevice, j->stream));
    GV_CK(cudaStreamSynchronize(j->stream));
    return GV_OK;
}

gv_status virt_update_trans(gv_job* j, int walker, int nset, const int32_t* hops, double* out)
{
    for (int i = 0; i < 4 * nset; ++i)
        if (hops[i] < -1 || hops[i] >= j->Ns) return GV_ERR_INVALID;
    const size_t nout = size_t(nset) * j->ch.Nexc * 2;
    int32_t* dh = nullptr;
    double* dout = nullptr;
    gv_status st = diag_pair(j, size_t(4) * nset, nout, &dh, &dout);
    if (st) return st;
    cudaError_t e = copy_async(dh, hops, sizeof(int32_t) * 4 * nset, cudaMemcpyHostToDevice, j->stream);
    const size_t sm = (j->cfg.precision == GV_PREC_FP64 ? sizeof(cx<double>) : sizeof(cx<float>)) * 2 * j->Nmax +
                      sizeof(double) * 6 * 4 + 16;
    if (!e) {
        if (j->cfg.precision == GV_PREC_FP64) k_virt_trans<double, 128><<<nset, 128, sm, j->stream>>>(j->d, walker, nset, dh, dout);
        else k_virt_trans<float, 128><<<nset, 128, sm, j->stream>>>(j->d, walker, nset, dh, dout);
        e = cudaGetLastError();
    }
    if (!e) e = copy_async(out, dout, sizeof(double) * nout, cudaMemcpyDeviceToHost, j->stream);
    if (!e) e = cudaStreamSynchronize(j->stream);
    return cuda_status(e);
}

constexpr double kMixedMaxInverse = 1e6;

// Largest |(A^-1)_ij| over both flavours of every walker (stored precision).
gv_status inverse_max_abs(gv_job* j, double* out)
{
    void* p = nullptr;
    gv_status st = diag_scratch(j, sizeof(double) * j->W, &p);
    if (st) return st;
    double* d = static_cast<double*>(p);
    if (j->cfg.precision == GV_PREC_FP64) k_inverse_max_abs<double, 256><<<j->W, 256, 0, j->stream>>>(j->d, d);
    else k_inverse_max_abs<float, 256><<<j->W, 256, 0, j->stream>>>(j->d, d);
    cudaError_t e = cudaGetLastError();
    if (!e) e = copy_async(out, d, sizeof(double) * j->W, cudaMemcpyDeviceToHost, j->stream);
    if (!e) e = cudaStreamSynchronize(j->stream);
    ++j->total_launches;
    return cuda_status(e);
}

// vmc.cpp:243-263 for the exciton channel: with every walker inverted in
// channel state 0, pick the state of largest |Amp| (first maximum; the
// overlaps come from the determinant lemma instead of one LU per state),
// replay the reference's hop path 0 -> 1 -> ... -> Nexc-1 -> kmax for the
// Fock-state slots and sign, invert in that state and set the weight.
gv_status trans_start(gv_job* j)
{
    const int W = j->W, Nexc = j->ch.Nexc;
    void* p = nullptr;
    gv_status st = diag_scratch(j, sizeof(double) * size_t(W) * Nexc, &p);
    if (st) return st;
    double* dov = static_cast<double*>(p);
    std::vector<double> ov(size_t(W) * Nexc);
    st = trans_overlaps(j, dov);
    if (!st && (copy_async(ov.data(), dov, ov.size() * sizeof(double), cudaMemcpyDeviceToHost, j->stream) ||
                cudaStreamSynchronize(j->stream)))
        st = GV_ERR_CUDA;
    if (st) return st;
    WavHost base = wav_state0(j);
    for (int k = 0; k < Nexc; ++k) wav_hop(j, base, k);
    std::vector<WavHost> ws(W, base);
    for (int w = 0; w < W; ++w) {
        int kmax = 0;
        double best = ov[size_t(w) * Nexc];
        for (int k = 1; k < Nexc; ++k)
            if (ov[size_t(w) * Nexc + k] > best) { best = ov[size_t(w) * Nexc + k]; kmax = k; }
        wav_hop(j, ws[w], kmax);
    }
    if ((st = upload_wav(j, ws))) return st;
    if ((st = invert_all(j))) return st;
    return trans_overlaps(j, nullptr);
}

// vmc.cpp:243-263 in the longitudinal channel: overlaps of every state from
// the walker's state-0 inverses and R (the determinant lemma, no LU per
// state), the first state of largest |Amp|, the reference's hop path
// 0 -> 1 -> ... -> Nexc-1 -> kmax replayed on the host (Slater rows, sign),
// then the inverses, R and the weight in that state.
gv_status long_start(gv_job* j)
{
    const int W = j->W, Nexc = j->ch.Nexc;
    void* p = nullptr;
    gv_status st = diag_scratch(j, sizeof(double) * size_t(W) * Nexc, &p);
    if (st) return st;
    double* dov = static_cast<double*>(p);
    std::vector<double> ov(size_t(W) * Nexc);
    st = long_states(j, dov);
    if (!st && (copy_async(ov.data(), dov, ov.size() * sizeof(double), cudaMemcpyDeviceToHost, j->stream) ||
                cudaStreamSynchronize(j->stream)))
        st = GV_ERR_CUDA;
    if (st) return st;
    WavHost base = wav_state0(j);
    for (int k = 0; k < Nexc; ++k) long_wav_hop(j, base, k);
    std::vector<WavHost> ws(W, base);
    for (int w = 0; w < W; ++w) {
        int kmax = 0;
        double best = ov[size_t(w) * Nexc];
        for (int k = 1; k < Nexc; ++k)
            if (ov[size_t(w) * Nexc + k] > best) { best = ov[size_t(w) * Nexc + k]; kmax = k; }
        long_wav_hop(j, ws[w], kmax);
    }
    if ((st = upload_wav(j, ws))) return st;
    if ((st = invert_all(j))) return st;
    return long_states(j, nullptr);
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
    GV_CK(copy_async(j->d.fock, fock.data(), fock.size() * sizeof(int16_t), cudaMemcpyHostToDevice, j->stream));
    GV_CK(copy_async(j->d.part, part.data(), part.size() * sizeof(int16_t), cudaMemcpyHostToDevice, j->stream));
    return GV_OK;
}

// ---- Checkpoint blob: header, then the device arrays below in this order,
// each copied whole.
constexpr char kCkptMagic[8] = {'G', 'V', 'C', 'K', 'P', 'T', '0', '1'};

struct CkptHeader {
    char magic[8];
    uint32_t header_bytes;
    int32_t flags;
    int32_t L, channel, q[2], precision, n_walkers, N[2], Nexc;
    uint32_t walker_base;
    uint64_t seed;
    double phi, neel, neel_exp, phase_shift[2], phi_range[2], neel_range[2];
    uint64_t payload_bytes;
    uint64_t checksum;   // FNV-1a 64 over the payload
};

struct CkptSection {
    void* dev;
    size_t bytes;
};

std::vector<CkptSection> ckpt_sections(gv_job* j, bool inverses)
{
    const size_t W = size_t(j->W), Ns = size_t(j->Ns), Nmax = size_t(j->Nmax);
    const DevJob& d = j->d;
    std::vector<CkptSection> s = {
        {d.fock, W * 2 * Ns * sizeof(int16_t)},
        {d.part, W * 2 * Nmax * sizeof(int16_t)},
        {d.amp_m, W * sizeof(cx<double>)},
        {d.amp_e, W * sizeof(int32_t)},
        {d.rng_next, W * sizeof(uint64_t)},
        {d.counts, W * 5 * sizeof(unsigned long long)},
        {d.since_reinv, W * sizeof(int32_t)},
        {d.checks, W * sizeof(unsigned long long)},
        {d.drift_seen, W * sizeof(double)},
        {d.status, W * sizeof(int32_t)},
        {d.pj, W * 2 * sizeof(cx<double>)},
        {d.pj_n, W * sizeof(int32_t)},
        {d.sm, W * sizeof(cx<double>)},
        {d.sm_n, W * sizeof(int32_t)},
        {d.ss, size_t(10) * Ns * Ns * sizeof(double)},
        {d.ss_n, sizeof(int32_t)},
    };
    const size_t Nexc = size_t(j->ch.Nexc);
    if (exc(j)) {
        s.push_back({d.worb, W * 2 * Nmax * sizeof(int16_t)});
        s.push_back({d.wslot, W * 2 * Ns * sizeof(int16_t)});
        s.push_back({d.cur, W * sizeof(int32_t)});
        s.push_back({d.wsign, W * sizeof(int32_t)});
        s.push_back({d.sigma, W * sizeof(double)});
        s.push_back({d.pjx, W * 2 * Nexc * Nexc * sizeof(cx<double>)});
        if (d.pxs) {
            s.push_back({d.pxs, W * kHoSlots * 3 * Nexc * sizeof(cx<float>)});
            s.push_back({d.pxs_n, W * sizeof(int32_t)});
        }
    }
    if (inverses) {
        const size_t es = j->cfg.precision == GV_PREC_FP64 ? sizeof(cx<double>) : sizeof(cx<float>);
        s.push_back({d.Ai[0], W * size_t(j->N[0]) * j->N[0] * es});
        s.push_back({d.Ai[1], W * size_t(j->N[1]) * j->N[1] * es});
        if (j->trans) {
            s.push_back({d.gup, W * size_t(j->N[0]) * Nexc * es});
            s.push_back({d.gdn, W * Nmax * es});
        }
        if (j->lng) s.push_back({d.gup, W * 2 * Nmax * size_t(Ns) * es});   // the overlap tables R
    }
    return s;
}

uint64_t fnv1a64(const unsigned char* p, size_t n)
{
    uint64_t h = 0xcbf29ce484222325ull;
    for (size_t i = 0; i < n; ++i) { h ^= p[i]; h *= 0x100000001b3ull; }
    return h;
}

CkptHeader ckpt_header(const gv_job* j, int flags)
{
    CkptHeader h;
    std::memset(&h, 0, sizeof(h));
    std::memcpy(h.magic, kCkptMagic, sizeof(h.magic));
    h.header_bytes = sizeof(CkptHeader);
    h.flags = flags;
    const gv_job_config& c = j->cfg;
    h.L = c.L; h.channel = c.channel; h.q[0] = c.q[0]; h.q[1] = c.q[1];
    h.precision = c.precision; h.n_walkers = c.n_walkers;
    h.N[0] = j->N[0]; h.N[1] = j->N[1]; h.Nexc = j->ch.Nexc;
    h.walker_base = c.walker_base; h.seed = c.seed;
    h.phi = c.phi; h.neel = c.neel; h.neel_exp = c.neel_exp;
    for (int i = 0; i < 2; ++i) {
        h.phase_shift[i] = c.phase_shift[i];
        h.phi_range[i] = c.phi_range[i];
        h.neel_range[i] = c.neel_range[i];
    }
    return h;
}

// The fields of two headers that must agree for a restore (the blob's
// precision only matters when it carries inverses).
bool ckpt_compatible(const CkptHeader& a, const CkptHeader& b)
{
    if (a.L != b.L || a.channel != b.channel || a.q[0] != b.q[0] || a.q[1] != b.q[1] ||
        a.n_walkers != b.n_walkers || a.N[0] != b.N[0] || a.N[1] != b.N[1] || a.Nexc != b.Nexc ||
        a.walker_base != b.walker_base || a.seed != b.seed)
        return false;
    if (a.phi != b.phi || a.neel != b.neel || a.neel_exp != b.neel_exp) return false;
    for (int i = 0; i < 2; ++i)
        if (a.phase_shift[i] != b.phase_shift[i] || a.phi_range[i] != b.phi_range[i] ||
            a.neel_range[i] != b.neel_range[i])
            return false;
    if ((a.flags & GV_CKPT_INVERSES) && a.precision != b.precision) return false;
    return true;
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
    if (channel != GV_CH_GROUNDSTATE && channel != GV_CH_TRANS && channel != GV_CH_LONG) return GV_ERR_INVALID;
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

gv_status gv_channel_states(int32_t L, const double* bc, int32_t channel, const int32_t* q, int32_t* exc_up,
                            int32_t* exc_dn)
{
    if (L < 4 || L > 32 || (L % 2) || !bc || !q || !exc_up || !exc_dn) return GV_ERR_INVALID;
    if (channel != GV_CH_TRANS && channel != GV_CH_LONG) return GV_ERR_INVALID;
    Orbitals o = make_orbitals(L, bc[0], bc[1]);
    if (!o.ok) return GV_ERR_INVALID;
    Channel ch = make_channel(o, channel, q[0], q[1]);
    if (channel == GV_CH_LONG) {
        if (!ch.ok) return GV_ERR_INVALID;
        for (int k = 0; k < ch.Nexc; ++k) { exc_up[k] = ch.exc_up[k]; exc_dn[k] = ch.exc_dn[k]; }
        return GV_OK;
    }
    std::vector<int16_t> up, dn;
    if (!ch.ok || !trans_tables(ch, up, dn)) return GV_ERR_INVALID;
    for (int k = 0; k < ch.Nexc; ++k) { exc_up[k] = up[k]; exc_dn[k] = dn[k]; }
    return GV_OK;
}

gv_status gv_fock_quantum_numbers(int32_t L, const double* bc, int32_t* out)
{
    if (L < 2 || L > 64 || (L % 2) || !bc || !out) return GV_ERR_INVALID;
    Orbitals o = make_orbitals(L, bc[0], bc[1]);
    if (!o.ok) return GV_ERR_INVALID;
    for (int i = 0; i < o.Nk; ++i)
        for (int band = 0; band < 2; ++band) {
            const int f = 2 * i + band;   // fock index: MBZ point i, band
            out[3 * f] = o.kx[i];
            out[3 * f + 1] = o.ky[i];
            out[3 * f + 2] = band;
        }
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

const char* gv_last_cuda_error(void) { return g_last_cuda_error; }

gv_status gv_transfer_bytes(uint64_t* h2d, uint64_t* d2h)
{
    if (h2d) *h2d = g_bytes_h2d.load();
    if (d2h) *d2h = g_bytes_d2h.load();
    return GV_OK;
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
        case GV_ERR_TOO_LARGE: return "size exceeds the entry point's fixed limit (gv_slater_invert_noalloc: N <= 128)";
        default: return "unknown status";
    }
}

gv_status gv_job_footprint(const gv_job_config* c, uint64_t* bytes)
{
    if (!valid_config(c) || !bytes) return GV_ERR_INVALID;
    const uint64_t Ns = uint64_t(c->L) * c->L, Nk = Ns / 2, W = c->n_walkers;
    const bool tr = c->channel == GV_CH_TRANS, lg = c->channel == GV_CH_LONG;
    const uint64_t N0 = tr ? Ns / 2 + 1 : Ns / 2, N1 = tr ? Ns / 2 - 1 : Ns / 2, Nmax = std::max(N0, N1);
    const uint64_t Nexc = tr ? Ns / 2 : lg ? Ns + 1 : 1;
    const uint64_t es = c->precision == GV_PREC_FP64 ? 16 : 8;
    uint64_t b = 0;
    b += Ns * Nk * (16 + 8);                 // phase tables
    b += W * 4 * Ns * (16 + 8);              // coefficients
    b += W * (N0 * N0 + N1 * N1) * es;       // inverses
    b += W * (2 * Ns + 2 * Nmax) * 2;        // occupancy
    b += W * 256;                            // per-walker scalars
    b += W * Nmax * Nmax * 16;               // FP64 re-inversion scratch
    b += 5 * Ns * Ns * 16;                   // StatSpinStruct sums
    b += 2 * Ns * ((W + 31) / 32) * 4;       // occupation bitsets
    b += Ns * Ns * 8;                        // FP32 staging sums of a tensor-core StatSpinStruct measurement
    if (tr) {
        b += W * (N0 * Nexc + Nmax) * es;    // overlap rows GupT and g
        b += W * (2 * Ns + 2 * Nmax) * 2;    // wavefunction Fock state
        b += W * 2 * Nexc * Nexc * 16;       // ProjHeis H and O sums
        if (c->precision == GV_PREC_MIXED) b += W * N1 * Nexc * 8;   // tensor-core overlap rows
    }
    if ((tr || lg) && c->precision != GV_PREC_FP64) {
        b += W * (uint64_t(kHoSlots) * 3 * Nexc * 8 + 4);   // FP32 factors of measurements waiting for their block
        const uint64_t per = 2 * Nexc * Nexc * 16;
        b += std::max<uint64_t>(1, std::min<uint64_t>(W, (uint64_t(32) << 20) / per)) * per;   // read-out scratch
    }
    if (lg) {
        b += W * 2 * Nmax * Ns * es;         // overlap table R of both flavours
        b += W * (2 * Ns + 2 * Nmax) * 2;    // wavefunction Fock state
        b += W * 2 * Nexc * Nexc * 16;       // ProjHeis H and O sums
        if (c->precision == GV_PREC_MIXED && Ns / 2 <= uint64_t(kTcM) && W * 2 * Ns * Ns * 8 <= (uint64_t(8) << 30))
            b += W * 2 * Ns * Ns * 8;        // tensor-core overlap sums of the bonds (upper-band orbitals)
    }
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
    j->ch = make_channel(j->orb, cfg->channel, cfg->q[0], cfg->q[1]);
    if (!j->ch.ok) { delete j; return GV_ERR_INVALID; }
    j->trans = cfg->channel == GV_CH_TRANS;
    j->lng = cfg->channel == GV_CH_LONG;
    if (j->trans && !trans_tables(j->ch, j->exu, j->exd)) { delete j; return GV_ERR_INVALID; }
    if (j->lng) {
        j->exu.assign(j->ch.exc_up.begin(), j->ch.exc_up.end());
        j->exd.assign(j->ch.exc_dn.begin(), j->ch.exc_dn.end());
    }
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
    // U_k / V_k of every walker (StagFluxWaveFunction.cpp:121-163): computed
    // once when the walkers share (phi, neel), else per walker on host threads
    // (each walker's table is the same whichever thread computes it).
    const size_t per_walker = size_t(4) * j->Ns;
    std::vector<cx<double>> cf64(size_t(j->W) * per_walker);
    std::vector<cx<float>> cf32(cf64.size());
    const bool shared = !(cfg->phi_range[1] > cfg->phi_range[0]) && !(cfg->neel_range[1] > cfg->neel_range[0]);
    auto fill = [&](int w) {
        std::vector<zd> c(per_walker);
        for (int fl = 0; fl < 2; ++fl)
            if (!stagflux_coefs(j->orb, j->wphi[w], j->wneel[w], cfg->neel_exp, fl, &c[size_t(fl) * 2 * j->Ns])) return false;
        for (size_t i = 0; i < per_walker; ++i) {
            cf64[size_t(w) * per_walker + i] = {c[i].real(), c[i].imag()};
            cf32[size_t(w) * per_walker + i] = {float(c[i].real()), float(c[i].imag())};
        }
        return true;
    };
    bool coef_ok = true;
    if (shared) {
        coef_ok = fill(0);
        for (int w = 1; coef_ok && w < j->W; ++w) {
            std::copy(cf64.begin(), cf64.begin() + per_walker, cf64.begin() + size_t(w) * per_walker);
            std::copy(cf32.begin(), cf32.begin() + per_walker, cf32.begin() + size_t(w) * per_walker);
        }
    } else {
        const int nth = std::max(1, std::min(16, int(std::thread::hardware_concurrency())));
        std::vector<std::thread> pool;
        std::atomic<bool> ok_all{true};
        for (int t = 0; t < nth; ++t)
            pool.emplace_back([&, t] {
                for (int w = t; w < j->W; w += nth)
                    if (!fill(w)) ok_all = false;
            });
        for (auto& th : pool) th.join();
        coef_ok = ok_all;
    }
    if (!coef_ok) {
        delete j;
        return GV_ERR_NAN;
    }
    std::vector<cx<double>> ph64(ph.size());
    std::vector<cx<float>> ph32(ph.size());
    for (size_t i = 0; i < ph.size(); ++i) {
        ph64[i] = {ph[i].real(), ph[i].imag()};
        ph32[i] = {float(ph[i].real()), float(ph[i].imag())};
    }
    std::vector<int32_t> edges(size_t(2) * j->Ns * 4);
    for (int e = 0; e < 2 * j->Ns; ++e) {
        const int a = j->lat.edge_i[e], b = j->lat.edge_j[e];
        int ka = 0, kb = 0;
        while (ka < 3 && j->lat.nbr[a * 4 + ka] != b) ++ka;
        while (kb < 3 && j->lat.nbr[b * 4 + kb] != a) ++kb;
        edges[4 * e] = a; edges[4 * e + 1] = b; edges[4 * e + 2] = ka; edges[4 * e + 3] = kb;
    }

    auto fail = [&](gv_status s) { gv_job_destroy(j); return s; };
    {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&j->n_sm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
            delete j;
            return GV_ERR_CUDA;
        }
    }
    if (cudaStreamCreateWithFlags(&j->stream, cudaStreamNonBlocking) != cudaSuccess) { delete j; return GV_ERR_CUDA; }
    if (statspin_tc_ok(j) &&   // created here: a measurement may run under stream capture
        (cudaStreamCreateWithFlags(&j->side, cudaStreamNonBlocking) != cudaSuccess ||
         cudaEventCreateWithFlags(&j->fork_ev, cudaEventDisableTiming) != cudaSuccess ||
         cudaEventCreateWithFlags(&j->join_ev, cudaEventDisableTiming) != cudaSuccess)) {
        if (j->side) cudaStreamDestroy(j->side);
        if (j->fork_ev) cudaEventDestroy(j->fork_ev);
        cudaStreamDestroy(j->stream);
        delete j;
        return GV_ERR_CUDA;
    }
    if (cudaEventCreate(&j->ev0) != cudaSuccess || cudaEventCreate(&j->ev1) != cudaSuccess) return fail(GV_ERR_CUDA);

    DevJob& d = j->d;
    d.L = L; d.Ns = j->Ns; d.Nk = j->Nk; d.Nexc = j->ch.Nexc; d.W = j->W;
    d.N[0] = j->N[0]; d.N[1] = j->N[1]; d.Nmax = j->Nmax;
    d.precision = cfg->precision; d.channel = cfg->channel;
    d.seed = cfg->seed; d.walker_base = cfg->walker_base; d.reinv_every = cfg->reinv_every;
    d.trace = nullptr; d.trace_walker = -1;
    d.wait_limit = kTcWaitLimit;
    d.forced_walker = -1; d.forced_v1 = d.forced_v2 = 0; d.forced_accept = 0; d.forced_khop = -1;
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
        (st = dalloc(j, &d.checks, size_t(j->W) * sizeof(unsigned long long))) ||
        (st = dalloc(j, &d.drift_seen, size_t(j->W) * sizeof(double))) ||
        (st = dalloc(j, &d.status, size_t(j->W) * sizeof(int32_t))) ||
        (st = dalloc(j, &d.pj, size_t(j->W) * 2 * sizeof(cx<double>))) ||
        (st = dalloc(j, &d.pj_n, size_t(j->W) * sizeof(int32_t))) ||
        (st = dalloc(j, &d.sm, size_t(j->W) * sizeof(cx<double>))) ||
        (st = dalloc(j, &d.sm_n, size_t(j->W) * sizeof(int32_t))) ||
        (st = dalloc(j, &d.ss, size_t(5) * j->Ns * j->Ns * 2 * sizeof(double))) ||
        (st = dalloc(j, &d.ss_n, sizeof(int32_t))) ||
        (st = dalloc(j, &d.occ, sizeof(uint32_t) * 2 * j->Ns * ((j->W + 31) / 32))) ||
        (st = dalloc(j, &d.ss32, sizeof(float2) * j->Ns * j->Ns)) ||
        (st = dalloc(j, &d.scratch64, scratch_walkers(j) * j->Nmax * j->Nmax * sizeof(cx<double>))))
        return fail(st);
    d.nbr = nbr; d.edges = reinterpret_cast<const int4*>(edg); d.phase64 = p64; d.phase32 = p32; d.coef64 = c64; d.coef32 = c32;
    d.Ai[0] = a0; d.Ai[1] = a1;
    d.worb = nullptr; d.wslot = nullptr; d.exc_up = nullptr; d.exc_dn = nullptr; d.cur = nullptr; d.wsign = nullptr;
    d.sigma = nullptr; d.gup = nullptr; d.gdn = nullptr; d.pjx = nullptr; d.zbuf = nullptr;
    d.pxs = nullptr; d.pxs_n = nullptr;
    d.track_sm = nullptr; d.track_lw = nullptr; d.track_n = nullptr; d.track_cap = 0;
    if (exc(j)) {
        const int Nexc = j->ch.Nexc;
        // overlap rows: GupT and g (transverse); R of both flavours over every orbital (longitudinal)
        const size_t gup = j->lng ? size_t(2) * j->Nmax * j->Ns : size_t(j->N[0]) * Nexc;
        int16_t *eu = nullptr, *ed = nullptr;
        if ((st = dalloc(j, &d.worb, size_t(j->W) * 2 * j->Nmax * sizeof(int16_t))) ||
            (st = dalloc(j, &d.wslot, size_t(j->W) * 2 * j->Ns * sizeof(int16_t))) ||
            (st = dalloc(j, &eu, size_t(Nexc) * sizeof(int16_t))) ||
            (st = dalloc(j, &ed, size_t(Nexc) * sizeof(int16_t))) ||
            (st = dalloc(j, &d.cur, size_t(j->W) * sizeof(int32_t))) ||
            (st = dalloc(j, &d.wsign, size_t(j->W) * sizeof(int32_t))) ||
            (st = dalloc(j, &d.sigma, size_t(j->W) * sizeof(double))) ||
            (st = dalloc(j, &d.gup, size_t(j->W) * gup * es)) ||
            (st = dalloc(j, &d.gdn, size_t(j->W) * j->Nmax * es)) ||
            (st = dalloc(j, &d.pjx, size_t(j->W) * 2 * Nexc * Nexc * sizeof(cx<double>))))
            return fail(st);
        if (trans_z_tc_ok(j) && (st = dalloc(j, &d.zbuf, size_t(j->W) * j->N[1] * Nexc * sizeof(cx<float>))))
            return fail(st);
        if (long_z_tc_ok(j) && (st = dalloc(j, &d.zbuf, size_t(j->W) * 2 * j->Ns * j->Ns * sizeof(cx<float>))))
            return fail(st);
        if (j->cfg.precision != GV_PREC_FP64 &&
            ((st = dalloc(j, &d.pxs, size_t(j->W) * kHoSlots * 3 * Nexc * sizeof(cx<float>))) ||
             (st = dalloc(j, &d.pxs_n, size_t(j->W) * sizeof(int32_t)))))
            return fail(st);
        d.exc_up = eu; d.exc_dn = ed;
        if (copy_async(eu, j->exu.data(), Nexc * sizeof(int16_t), cudaMemcpyHostToDevice, j->stream) ||
            copy_async(ed, j->exd.data(), Nexc * sizeof(int16_t), cudaMemcpyHostToDevice, j->stream))
            return fail(GV_ERR_CUDA);
    }
    if (copy_async(nbr, j->lat.nbr.data(), sizeof(int32_t) * 4 * j->Ns, cudaMemcpyHostToDevice, j->stream) ||
        copy_async(edg, edges.data(), edges.size() * sizeof(int32_t), cudaMemcpyHostToDevice, j->stream) ||
        copy_async(p64, ph64.data(), ph64.size() * sizeof(cx<double>), cudaMemcpyHostToDevice, j->stream) ||
        copy_async(p32, ph32.data(), ph32.size() * sizeof(cx<float>), cudaMemcpyHostToDevice, j->stream) ||
        copy_async(c64, cf64.data(), cf64.size() * sizeof(cx<double>), cudaMemcpyHostToDevice, j->stream) ||
        copy_async(c32, cf32.data(), cf32.size() * sizeof(cx<float>), cudaMemcpyHostToDevice, j->stream) ||
        cudaStreamSynchronize(j->stream))
        return fail(GV_ERR_CUDA);
    *out = j;
    return GV_OK;
}

gv_status gv_job_destroy(gv_job* j)
{
    if (!j) return GV_OK;
    if (j->stream) cudaStreamSynchronize(j->stream);
    for (auto& kv : j->graphs) cudaGraphExecDestroy(kv.second.exec);
    for (void* p : j->allocs) cudaFree(p);
    cudaFree(j->diag);
    cudaFree(j->d.track_sm);
    cudaFree(j->d.track_lw);
    cudaFree(j->d.track_n);
    if (j->ev0) cudaEventDestroy(j->ev0);
    for (cudaEvent_t e : j->ev_pool) cudaEventDestroy(e);
    if (j->tev0) cudaEventDestroy(j->tev0);
    if (j->tev1) cudaEventDestroy(j->tev1);
    if (j->ev1) cudaEventDestroy(j->ev1);
    if (j->stream) cudaStreamDestroy(j->stream);
    if (j->side) cudaStreamDestroy(j->side);
    if (j->fork_ev) cudaEventDestroy(j->fork_ev);
    if (j->join_ev) cudaEventDestroy(j->join_ev);
    delete j;
    return GV_OK;
}

gv_status gv_job_dims(const gv_job* j, int32_t* Ns, int32_t* Nup, int32_t* Ndn, int32_t* Nexc)
{
    if (!j) return GV_ERR_INVALID;
    if (Ns) *Ns = j->Ns;
    if (Nup) *Nup = j->N[0];
    if (Ndn) *Ndn = j->N[1];
    if (Nexc) *Nexc = j->ch.Nexc;
    return GV_OK;
}

gv_status gv_job_set_meas_mask(gv_job* j, int32_t mask)
{
    if (!j || (mask & ~(GV_MEAS_PROJHEIS | GV_MEAS_STAGMAGN | GV_MEAS_STATSPIN | kTrackMask))) return GV_ERR_INVALID;
    j->cfg.meas_mask = mask;
    return GV_OK;
}

static gv_status reset_quantities(gv_job* j)
{
    GV_CK(cudaMemsetAsync(j->d.pj, 0, sizeof(cx<double>) * 2 * j->W, j->stream));
    GV_CK(cudaMemsetAsync(j->d.pj_n, 0, sizeof(int32_t) * j->W, j->stream));
    GV_CK(cudaMemsetAsync(j->d.sm, 0, sizeof(cx<double>) * j->W, j->stream));
    GV_CK(cudaMemsetAsync(j->d.sm_n, 0, sizeof(int32_t) * j->W, j->stream));
    GV_CK(cudaMemsetAsync(j->d.ss, 0, sizeof(double) * 10 * j->Ns * j->Ns, j->stream));
    GV_CK(cudaMemsetAsync(j->d.ss_n, 0, sizeof(int32_t), j->stream));
    GV_CK(cudaMemsetAsync(j->d.ss32, 0, sizeof(float2) * j->Ns * j->Ns, j->stream));
    if (exc(j))
        GV_CK(cudaMemsetAsync(j->d.pjx, 0, sizeof(cx<double>) * 2 * size_t(j->W) * j->ch.Nexc * j->ch.Nexc, j->stream));
    if (j->d.pxs_n) GV_CK(cudaMemsetAsync(j->d.pxs_n, 0, sizeof(int32_t) * j->W, j->stream));
    if (j->d.track_n) GV_CK(cudaMemsetAsync(j->d.track_n, 0, sizeof(int32_t) * j->W, j->stream));
    return GV_OK;
}

gv_status gv_job_reset_quantities(gv_job* j)
{
    if (!j) return GV_ERR_INVALID;
    return reset_quantities(j);
}

gv_status gv_job_measure(gv_job* j)
{
    if (!j) return GV_ERR_INVALID;
    if (!j->ready) return GV_ERR_NOT_READY;
    const int mask = j->cfg.meas_mask;
    gv_status st = GV_OK;
    const bool tcph = (j->cfg.flags & GV_FLAG_TC_PROJHEIS) && (mask & GV_MEAS_PROJHEIS);
    const int inner = mask & kInnerMask & (tcph ? ~GV_MEAS_PROJHEIS : ~0);
    const int pairs = ((mask & GV_MEAS_STATSPIN) ? 1 : 0) | (tcph ? 2 : 0);
    if (inner)
        st = j->trans ? measure_trans_dispatch(j, inner)
             : j->lng ? measure_long_dispatch(j, inner) : walk_dispatch(j, 0, 0, 1, inner, 1);
    if (!st && pairs) st = statspin_dispatch(j, pairs);
    if (!st && (mask & kTrackMask)) st = tracks_dispatch(j, mask);
    return st ? st : gv_job_synchronize(j);
}

gv_status gv_job_set_wait_limit(gv_job* j, int32_t polls)
{
    if (!j) return GV_ERR_INVALID;
    GV_CK(cudaStreamSynchronize(j->stream));
    j->d.wait_limit = polls < 0 ? kTcWaitLimit : polls;
    for (auto& kv : j->graphs) cudaGraphExecDestroy(kv.second.exec);   // they hold the old limit
    j->graphs.clear();
    return GV_OK;
}

gv_status gv_job_read_drift_checks(gv_job* j, double* drift, uint64_t* checks)
{
    if (!j) return GV_ERR_INVALID;
    GV_CK(cudaStreamSynchronize(j->stream));
    if (drift) GV_CK(copy_sync(drift, j->d.drift_seen, sizeof(double) * j->W, cudaMemcpyDeviceToHost));
    if (checks) GV_CK(copy_sync(checks, j->d.checks, sizeof(uint64_t) * j->W, cudaMemcpyDeviceToHost));
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
    GV_CK(cudaMemsetAsync(j->d.checks, 0, sizeof(unsigned long long) * W, j->stream));
    GV_CK(cudaMemsetAsync(j->d.drift_seen, 0, sizeof(double) * W, j->stream));
    // vmc.cpp:221-241: up to 10 random starts until the amplitude is non-zero.
    // A mixed-precision job also redraws a random start whose inverse (in the
    // picked channel state) has an entry above kMixedMaxInverse: such a
    // configuration's amplitude is many orders below its neighbours', and its
    // FP32 ratios would overflow or cancel to noise on the first step.
    const bool screen = j->cfg.precision == GV_PREC_MIXED && !up;
    std::vector<double> amax(W);
    for (int attempt = 0; attempt < 10; ++attempt) {
        if (exc(j)) {   // every walker starts in channel state 0
            gv_status st = upload_wav(j, std::vector<WavHost>(W, wav_state0(j)));
            if (st) return st;
        }
        gv_status st = upload_configs(j, cfg);
        if (st) return st;
        st = invert_all(j);
        if (st) return st;
        GV_CK(copy_async(status.data(), j->d.status, sizeof(int32_t) * W, cudaMemcpyDeviceToHost, j->stream));
        GV_CK(cudaStreamSynchronize(j->stream));
        bool again = false;
        for (int w = 0; w < W; ++w)
            if (status[w] == GV_ERR_SINGULAR && !up) { ran_init(j, w, &cfg[size_t(w) * Ns]); again = true; }
        if (!again && exc(j)) {
            for (int w = 0; w < W; ++w)
                if (status[w] != GV_OK) { j->ready = true; return status[w]; }
            if ((st = j->trans ? trans_start(j) : long_start(j))) return st;
        }
        if (!again && screen) {
            if ((st = inverse_max_abs(j, amax.data()))) return st;
            for (int w = 0; w < W; ++w)
                if (status[w] == GV_OK && !(amax[w] <= kMixedMaxInverse)) {
                    ran_init(j, w, &cfg[size_t(w) * Ns]);
                    again = true;
                }
        }
        if (!again) break;
        if (attempt == 9) return GV_ERR_SINGULAR;
        GV_CK(cudaMemsetAsync(j->d.status, 0, sizeof(int32_t) * W, j->stream));
    }
    for (int w = 0; w < W; ++w)
        if (status[w] != GV_OK) { j->ready = true; return status[w]; }
    j->ready = true;
    return exc(j) ? gv_job_synchronize(j) : GV_OK;
}

// The kernels of one MetroMC::Walk(len, meas) call, enqueued on the job's stream.
static gv_status enqueue_walk(gv_job* j, uint64_t len, uint64_t meas, int mask, gv_trace* dtrace, bool reset)
{
    if (meas && reset) {
        gv_status rs = reset_quantities(j);
        if (rs) return rs;
    }
    gv_status st = GV_OK;
    // GV_FLAG_TC_PROJHEIS: ProjHeis from the tensor-core pair pass instead of inside the walk
    const bool tcph = (j->cfg.flags & GV_FLAG_TC_PROJHEIS) && (mask & GV_MEAS_PROJHEIS);
    const int inner = mask & kInnerMask & (tcph ? ~GV_MEAS_PROJHEIS : ~0);
    const int pairs = ((mask & GV_MEAS_STATSPIN) ? 1 : 0) | (tcph ? 2 : 0);
    // the exciton walks measure in kernels of their own, between walk launches
    auto exc_walk = [&](uint64_t n) { return j->trans ? walk_trans_dispatch(j, n) : walk_long_dispatch(j, n); };
    if (!(mask & (GV_MEAS_STATSPIN | kTrackMask)) && !(exc(j) && mask) && !tcph) {
        st = exc(j) ? exc_walk(len) : walk_dispatch(j, len, 0, meas, mask);
    } else {
        // Split at the measurement points: steps [a, m] then measure after step m.
        uint64_t a = 0;
        while (a < len && !st) {
            uint64_t m = (a == 0) ? 0 : ((a + meas - 1) / meas) * meas;   // next s with s % meas == 0, s >= a
            if (j->d.trace) j->d.trace = dtrace + a;
            if (m >= len) {
                st = exc(j) ? exc_walk(len - a) : walk_dispatch(j, len - a, a, 0, 0);
                a = len;
                break;
            }
            const uint64_t nsteps = m - a + 1;
            if (exc(j)) {
                st = exc_walk(nsteps);
                if (!st && inner) st = j->trans ? measure_trans_dispatch(j, inner) : measure_long_dispatch(j, inner);
            } else {
                // ground state: ProjHeis / StagMagnZ inside the walk kernel at step m
                st = walk_dispatch(j, nsteps, a, meas, inner);
            }
            if (!st && pairs) st = statspin_dispatch(j, pairs);
            if (!st && (mask & kTrackMask)) st = tracks_dispatch(j, mask);
            a = m + 1;
        }
        j->d.trace = dtrace;
    }
    if (!st && (j->cfg.flags & GV_FLAG_REINV_DEFERRED) && j->cfg.reinv_every > 0) st = deferred_reinversion(j);
    return st;
}

// GV_FLAG_CUDA_GRAPHS: a walk call's kernels captured once per (len, meas,
// mask, reset) into a CUDA graph and replayed (kernel arguments are fixed per
// job: device pointers, step counts, the measurement mask).  A capture the
// runtime refuses turns the job's graphs off and enqueues the kernels directly.
static gv_status walk_graph(gv_job* j, uint64_t len, uint64_t meas, int mask, bool reset)
{
    const auto key = std::make_tuple(len, meas, mask, reset);
    auto it = j->graphs.find(key);
    if (it == j->graphs.end()) {
        const int64_t l0 = j->total_launches, ll0 = j->last_launches;
        GV_CK(cudaStreamBeginCapture(j->stream, cudaStreamCaptureModeThreadLocal));
        gv_status st = enqueue_walk(j, len, meas, mask, nullptr, reset);
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamEndCapture(j->stream, &g);
        const int64_t n = j->total_launches - l0;
        j->total_launches = l0;
        j->last_launches = ll0;
        if (st || e != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            cudaGetLastError();
            j->graphs_off = true;
            return enqueue_walk(j, len, meas, mask, nullptr, reset);
        }
        cudaGraphExec_t x = nullptr;
        e = cudaGraphInstantiate(&x, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            cudaGetLastError();
            j->graphs_off = true;
            return enqueue_walk(j, len, meas, mask, nullptr, reset);
        }
        if (j->graphs.size() >= 16) {
            for (auto& kv : j->graphs) cudaGraphExecDestroy(kv.second.exec);
            j->graphs.clear();
        }
        it = j->graphs.emplace(key, gv_job::WalkGraph{x, n}).first;
    }
    GV_CK(cudaGraphLaunch(it->second.exec, j->stream));
    j->last_launches += it->second.launches;
    j->total_launches += it->second.launches;
    ++j->graph_replays;
    return GV_OK;
}

static gv_status walk_impl(gv_job* j, uint64_t len, uint64_t meas, gv_trace* dtrace, int trace_walker,
                           bool reset = true)
{
    if (!j) return GV_ERR_INVALID;
    if (!j->ready) return GV_ERR_NOT_READY;
    const int mask = meas ? j->cfg.meas_mask : 0;
    j->d.trace = dtrace;
    j->d.trace_walker = trace_walker;
    j->last_launches = 0;
    GV_CK(cudaEventRecord(j->ev0, j->stream));
    const bool graph = (j->cfg.flags & GV_FLAG_CUDA_GRAPHS) && !j->graphs_off && !dtrace && !j->timing;
    gv_status st = graph ? walk_graph(j, len, meas, mask, reset) : enqueue_walk(j, len, meas, mask, dtrace, reset);
    GV_CK(cudaEventRecord(j->ev1, j->stream));
    j->d.trace = nullptr;
    j->d.trace_walker = -1;
    return st;
}

gv_status gv_job_walk(gv_job* j, uint64_t len, uint64_t meas) { return walk_impl(j, len, meas, nullptr, -1); }

gv_status gv_job_walk_continue(gv_job* j, uint64_t len, uint64_t meas)
{
    return walk_impl(j, len, meas, nullptr, -1, false);
}

gv_status gv_job_stream(gv_job* j, void** stream)
{
    if (!j || !stream) return GV_ERR_INVALID;
    *stream = j->stream;
    return GV_OK;
}

gv_status gv_job_walk_traced(gv_job* j, uint64_t len, uint64_t meas, int32_t walker, gv_trace* trace)
{
    if (!j || !trace || walker < 0 || walker >= j->W) return GV_ERR_INVALID;
    void* p = nullptr;
    gv_status st = diag_scratch(j, sizeof(gv_trace) * (len ? len : 1), &p);
    if (st) return st;
    gv_trace* dt = static_cast<gv_trace*>(p);
    st = walk_impl(j, len, meas, dt, walker);
    if (!st) {
        if (copy_async(trace, dt, sizeof(gv_trace) * len, cudaMemcpyDeviceToHost, j->stream) ||
            cudaStreamSynchronize(j->stream))
            st = GV_ERR_CUDA;
    }
    return st ? st : gv_job_synchronize(j);
}

// ---- Single-walker stepping: LatticeStepper::trystep / step, MetroMC::YesNo ----
// One streaming walk launch that runs walker w only, on the given proposal
// (v1, v2): accept = 0 evaluates it (ratio and arg-max channel state into
// *rec) and changes nothing; accept = 1 applies it with channel state khop
// (-1: the arg-max), exactly as an accepted step of gv_job_walk.
static gv_status forced_walk(gv_job* j, int w, int v1, int v2, int accept, int khop, gv_trace* rec)
{
    if (!j->step_trace) {
        gv_status st = dalloc(j, &j->step_trace, sizeof(gv_trace));
        if (st) return st;
    }
    DevJob& d = j->d;
    d.forced_walker = w; d.forced_v1 = v1; d.forced_v2 = v2; d.forced_accept = accept; d.forced_khop = khop;
    d.trace = j->step_trace;
    d.trace_walker = w;
    const bool fp64 = j->cfg.precision == GV_PREC_FP64;
    gv_status st;
    if (j->trans) st = fp64 ? launch_walk_trans<double>(j, 1) : launch_walk_trans<float>(j, 1);
    else if (j->lng) st = fp64 ? launch_walk_long<double>(j, 1) : launch_walk_long<float>(j, 1);
    else if (j->nt == 128) st = fp64 ? launch_walk<double, 128, 0>(j, 1, 0, 0, 0, 0) : launch_walk<float, 128, 0>(j, 1, 0, 0, 0, 0);
    else st = fp64 ? launch_walk<double, 256, 0>(j, 1, 0, 0, 0, 0) : launch_walk<float, 256, 0>(j, 1, 0, 0, 0, 0);
    d.forced_walker = -1;
    d.forced_khop = -1;
    d.trace = nullptr;
    d.trace_walker = -1;
    if (st) return st;
    if (rec) GV_CK(copy_async(rec, j->step_trace, sizeof(gv_trace), cudaMemcpyDeviceToHost, j->stream));
    GV_CK(cudaStreamSynchronize(j->stream));
    int32_t status = GV_OK;
    GV_CK(copy_sync(&status, j->d.status + w, sizeof(int32_t), cudaMemcpyDeviceToHost));
    return status;
}

// |Amp|^2 sigma of walker w (LatticeStepper::weight) as mantissa * 2^e2.
static gv_status walker_weight(gv_job* j, int w, double* mant, int32_t* e2)
{
    cx<double> m;
    int32_t e = 0;
    double sigma = 1.0;
    GV_CK(cudaStreamSynchronize(j->stream));
    GV_CK(copy_sync(&m, j->d.amp_m + w, sizeof(m), cudaMemcpyDeviceToHost));
    GV_CK(copy_sync(&e, j->d.amp_e + w, sizeof(e), cudaMemcpyDeviceToHost));
    if (exc(j)) GV_CK(copy_sync(&sigma, j->d.sigma + w, sizeof(double), cudaMemcpyDeviceToHost));
    int k = 0;
    *mant = std::frexp((m.x * m.x + m.y * m.y) * sigma, &k);
    *e2 = 2 * e + k;
    return GV_OK;
}

static gv_status walker_rng(gv_job* j, int w, uint64_t* k)
{
    GV_CK(cudaStreamSynchronize(j->stream));
    GV_CK(copy_sync(k, j->d.rng_next + w, sizeof(uint64_t), cudaMemcpyDeviceToHost));
    return GV_OK;
}

gv_status gv_job_stepper_weight(gv_job* j, int32_t walker, double* mant, int32_t* exp2)
{
    if (!j || !mant || !exp2 || walker < 0 || walker >= j->W) return GV_ERR_INVALID;
    if (!j->ready) return GV_ERR_NOT_READY;
    return walker_weight(j, walker, mant, exp2);
}

gv_status gv_job_trystep(gv_job* j, int32_t walker, int32_t* v, double* weight_mant, int32_t* weight_exp2,
                         int32_t* khop)
{
    if (!j || walker < 0 || walker >= j->W) return GV_ERR_INVALID;
    if (!j->ready) return GV_ERR_NOT_READY;
    uint64_t k = 0;
    gv_status st = walker_rng(j, walker, &k);
    if (st) return st;
    // u1 -> vertex, u2 -> neighbour slot (LatticeStepper.cpp:45-47), integer-exact as in the walk kernels
    uint32_t x[4];
    philox_call(j->cfg.seed, j->cfg.walker_base + uint32_t(walker), 0, k >> 1, x);
    const int v1 = scaled_floor(uint32_t(j->Ns), u52(x[0], x[1]));
    const int v2 = j->lat.nbr[size_t(v1) * 4 + int(u52(x[2], x[3]) >> 50)];
    gv_trace t{};
    st = forced_walk(j, walker, v1, v2, 0, -1, &t);
    if (st) return st;
    double m = 0.0;
    int32_t e2 = 0;
    st = walker_weight(j, walker, &m, &e2);
    if (st) return st;
    if (t.kind) {   // the proposal's weight: its ratio times the current weight
        int kk = 0;
        m = std::frexp(m * t.ratio, &kk);
        e2 += kk;
    }
    j->pend.w = walker;
    j->pend.v1 = v1;
    j->pend.v2 = v2;
    j->pend.khop = t.kind ? t.khop : -1;
    if (v) { v[0] = v1; v[1] = v2; }
    if (weight_mant) *weight_mant = m;
    if (weight_exp2) *weight_exp2 = e2;
    if (khop) *khop = j->pend.khop;
    return GV_OK;
}

gv_status gv_job_yesno(gv_job* j, int32_t walker, double ratio, int32_t* accepted)
{
    if (!j || !accepted || walker < 0 || walker >= j->W) return GV_ERR_INVALID;
    if (!j->ready) return GV_ERR_NOT_READY;
    uint64_t k = 0;
    gv_status st = walker_rng(j, walker, &k);
    if (st) return st;
    // u4, the step's fourth uniform (MetroMC.cpp:41); the stream then moves to the next step
    const double u4 = uniform_at(j->cfg.seed, j->cfg.walker_base + uint32_t(walker), 0, k + 3);
    const int acc = ratio > 1.0 ? (u4 < 1.0) : (u4 < ratio);
    const uint64_t next = k + 4;
    GV_CK(copy_sync(j->d.rng_next + walker, &next, sizeof(uint64_t), cudaMemcpyHostToDevice));
    if (!acc) {   // a rejected step: counted here (an accepted one by gv_job_step)
        uint64_t c[5];
        GV_CK(copy_sync(c, j->d.counts + size_t(walker) * 5, sizeof(c), cudaMemcpyDeviceToHost));
        c[0] += 1;
        c[3] += 1;
        GV_CK(copy_sync(j->d.counts + size_t(walker) * 5, c, sizeof(c), cudaMemcpyHostToDevice));
        if (j->pend.w == walker) j->pend.w = -1;
    }
    *accepted = acc;
    return GV_OK;
}

gv_status gv_job_step(gv_job* j, int32_t walker)
{
    if (!j || walker < 0 || walker >= j->W) return GV_ERR_INVALID;
    if (!j->ready) return GV_ERR_NOT_READY;
    if (j->pend.w != walker) return GV_ERR_INVALID;   // no evaluated proposal for this walker
    const gv_job::Pending p = j->pend;
    j->pend.w = -1;
    gv_status st = forced_walk(j, walker, p.v1, p.v2, 1, p.khop, nullptr);
    if (!st && (j->cfg.flags & GV_FLAG_REINV_DEFERRED) && j->cfg.reinv_every > 0) {
        st = deferred_reinversion(j);
        if (!st) st = gv_job_synchronize(j);
    }
    return st;
}

gv_status gv_job_update(gv_job* j, int32_t walker, const int32_t* hop, int32_t state)
{
    if (!j || !hop || walker < 0 || walker >= j->W) return GV_ERR_INVALID;
    if (!j->ready) return GV_ERR_NOT_READY;
    for (int i = 0; i < 4; ++i)
        if (hop[i] < -1 || hop[i] >= j->Ns) return GV_ERR_INVALID;
    if (hop[0] < 0 && hop[1] < 0 && hop[2] < 0 && hop[3] < 0) return GV_OK;   // the empty hop set
    // a nearest-neighbour exchange: flavour 0 from a to b, flavour 1 from b to a
    if (hop[0] < 0 || hop[1] < 0 || hop[2] != hop[1] || hop[3] != hop[0]) return GV_ERR_INVALID;
    if (state < -1 || state >= j->ch.Nexc) return GV_ERR_INVALID;
    std::vector<int16_t> fock(2 * size_t(j->Ns));
    GV_CK(cudaStreamSynchronize(j->stream));
    GV_CK(copy_sync(fock.data(), j->d.fock + size_t(walker) * 2 * j->Ns, fock.size() * sizeof(int16_t),
                    cudaMemcpyDeviceToHost));
    if (fock[hop[0]] < 0 || fock[j->Ns + hop[1]] < 0) return GV_ERR_INVALID;   // the hop's particles are absent
    if (j->pend.w == walker) j->pend.w = -1;
    return forced_walk(j, walker, hop[0], hop[1], 1, state, nullptr);
}

gv_status gv_job_synchronize(gv_job* j)
{
    if (!j) return GV_ERR_INVALID;
    GV_CK(cudaStreamSynchronize(j->stream));
    float ms = 0;
    if (cudaEventElapsedTime(&ms, j->ev0, j->ev1) == cudaSuccess) j->last_ms = ms;
    else cudaGetLastError();   // no walk recorded yet: clear the (non-sticky) error
    std::vector<int32_t> status(j->W);
    GV_CK(copy_sync(status.data(), j->d.status, sizeof(int32_t) * j->W, cudaMemcpyDeviceToHost));
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
    j->timing = true;
    j->ev_used.clear();
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
    j->timing = false;
    for (int q = 0; q < 3; ++q) { j->kind_ms[q] = 0.0; j->kind_n[q] = 0; j->kind_each[q].clear(); }
    for (auto& u : j->ev_used) {
        float t = 0;
        GV_CK(cudaEventElapsedTime(&t, j->ev_pool[u.second], j->ev_pool[u.second + 1]));
        j->kind_ms[u.first] += t;
        j->kind_n[u.first] += 1;
        j->kind_each[u.first].push_back(t);
    }
    return GV_OK;
}

gv_status gv_job_kernel_ms(gv_job* j, int32_t kind, double* ms, int64_t* launches)
{
    if (!j || kind < 0 || kind > 2) return GV_ERR_INVALID;
    if (ms) *ms = j->kind_ms[kind];
    if (launches) *launches = j->kind_n[kind];
    return GV_OK;
}

gv_status gv_job_kernel_times(gv_job* j, int32_t kind, double* out, int64_t capacity, int64_t* n)
{
    if (!j || kind < 0 || kind > 2 || (capacity > 0 && !out)) return GV_ERR_INVALID;
    const auto& v = j->kind_each[kind];
    const int64_t m = std::min<int64_t>(capacity, int64_t(v.size()));
    for (int64_t i = 0; i < m; ++i) out[i] = v[i];
    if (n) *n = int64_t(v.size());
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
    void* p = nullptr;
    gv_status st = diag_scratch(j, sizeof(double) * 2 * j->W, &p);
    if (st) return st;
    double* d = static_cast<double*>(p);
    if (j->cfg.precision == GV_PREC_FP64) k_drift<double, 256><<<dim3(j->W, 2), 256, 0, j->stream>>>(j->d, d);
    else k_drift<float, 256><<<dim3(j->W, 2), 256, 0, j->stream>>>(j->d, d);
    cudaError_t e = cudaGetLastError();
    if (!e) e = copy_async(out, d, sizeof(double) * 2 * j->W, cudaMemcpyDeviceToHost, j->stream);
    if (!e) e = cudaStreamSynchronize(j->stream);
    return cuda_status(e);
}

gv_status gv_job_virt_update(gv_job* j, int32_t walker, int32_t nset, const int32_t* hops, double* out)
{
    if (!j || !hops || !out || walker < 0 || walker >= j->W || nset < 0) return GV_ERR_INVALID;
    if (!j->ready) return GV_ERR_NOT_READY;
    if (j->trans) return virt_update_trans(j, walker, nset, hops, out);
    if (j->lng) return virt_update_long(j, walker, nset, hops, out);
    if (nset == 0) return GV_OK;
    for (int i = 0; i < 4 * nset; ++i)
        if (hops[i] < -1 || hops[i] >= j->Ns) return GV_ERR_INVALID;
    int32_t* dh = nullptr;
    double* dout = nullptr;
    gv_status st = diag_pair(j, size_t(4) * nset, size_t(2) * nset, &dh, &dout);
    if (st) return st;
    cudaError_t e = copy_async(dh, hops, sizeof(int32_t) * 4 * nset, cudaMemcpyHostToDevice, j->stream);
    const int per = 4;
    if (!e) {
        if (j->cfg.precision == GV_PREC_FP64)
            k_virt_update<double><<<(nset + per - 1) / per, 32 * per, 0, j->stream>>>(j->d, walker, nset, dh, dout);
        else
            k_virt_update<float><<<(nset + per - 1) / per, 32 * per, 0, j->stream>>>(j->d, walker, nset, dh, dout);
        e = cudaGetLastError();
    }
    if (!e) e = copy_async(out, dout, sizeof(double) * 2 * nset, cudaMemcpyDeviceToHost, j->stream);
    if (!e) e = cudaStreamSynchronize(j->stream);
    return cuda_status(e);
}

gv_status gv_job_read_config(gv_job* j, int8_t* up)
{
    if (!j || !up) return GV_ERR_INVALID;
    GV_CK(cudaStreamSynchronize(j->stream));
    std::vector<int16_t> fock(size_t(j->W) * 2 * j->Ns);
    GV_CK(copy_sync(fock.data(), j->d.fock, fock.size() * sizeof(int16_t), cudaMemcpyDeviceToHost));
    for (int w = 0; w < j->W; ++w)
        for (int v = 0; v < j->Ns; ++v) up[size_t(w) * j->Ns + v] = fock[size_t(w) * 2 * j->Ns + v] >= 0 ? 1 : 0;
    return GV_OK;
}

gv_status gv_job_read_particles(gv_job* j, int32_t walker, int32_t fl, int32_t* out)
{
    if (!j || !out || walker < 0 || walker >= j->W || fl < 0 || fl > 1) return GV_ERR_INVALID;
    GV_CK(cudaStreamSynchronize(j->stream));
    std::vector<int16_t> part(j->Nmax);
    GV_CK(copy_sync(part.data(), j->d.part + (size_t(walker) * 2 + fl) * j->Nmax, sizeof(int16_t) * j->Nmax,
                     cudaMemcpyDeviceToHost));
    for (int p = 0; p < j->N[fl]; ++p) out[p] = part[p];
    return GV_OK;
}

gv_status gv_job_read_amplitude(gv_job* j, double* mant, int32_t* exp10)
{
    if (!j || !mant || !exp10) return GV_ERR_INVALID;
    GV_CK(cudaStreamSynchronize(j->stream));
    std::vector<cx<double>> m(j->W);
    std::vector<int32_t> e(j->W), sg(j->W, 1);
    GV_CK(copy_sync(m.data(), j->d.amp_m, sizeof(cx<double>) * j->W, cudaMemcpyDeviceToHost));
    GV_CK(copy_sync(e.data(), j->d.amp_e, sizeof(int32_t) * j->W, cudaMemcpyDeviceToHost));
    if (exc(j)) GV_CK(copy_sync(sg.data(), j->d.wsign, sizeof(int32_t) * j->W, cudaMemcpyDeviceToHost));
    for (int w = 0; w < j->W; ++w) m[w] = m[w] * double(sg[w]);   // SlaterDeterminant::Amp (SlaterDeterminant.cpp:94)
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
    // AiT[f][p] = (A^-1)(p, f) is the reference's column-major m_mati[p + f*N].
    if (j->cfg.precision == GV_PREC_FP64) {
        GV_CK(copy_sync(out, static_cast<cx<double>*>(j->d.Ai[fl]) + size_t(walker) * n, n * sizeof(cx<double>),
                         cudaMemcpyDeviceToHost));
    } else {
        std::vector<cx<float>> a(n);
        GV_CK(copy_sync(a.data(), static_cast<cx<float>*>(j->d.Ai[fl]) + size_t(walker) * n, n * sizeof(cx<float>),
                         cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < n; ++i) { out[2 * i] = a[i].x; out[2 * i + 1] = a[i].y; }
    }
    return GV_OK;
}

gv_status gv_job_read_counts(gv_job* j, uint64_t* counts)
{
    if (!j || !counts) return GV_ERR_INVALID;
    GV_CK(cudaStreamSynchronize(j->stream));
    GV_CK(copy_sync(counts, j->d.counts, sizeof(uint64_t) * 5 * j->W, cudaMemcpyDeviceToHost));
    return GV_OK;
}

gv_status gv_job_read_state_index(gv_job* j, int32_t* state)
{
    if (!j || !state) return GV_ERR_INVALID;
    if (!exc(j)) {
        for (int w = 0; w < j->W; ++w) state[w] = 0;
        return GV_OK;
    }
    GV_CK(cudaStreamSynchronize(j->stream));
    GV_CK(copy_sync(state, j->d.cur, sizeof(int32_t) * j->W, cudaMemcpyDeviceToHost));
    return GV_OK;
}

gv_status gv_job_read_projheis(gv_job* j, double* vals, int32_t* nmeas)
{
    if (!j || !vals) return GV_ERR_INVALID;
    GV_CK(cudaStreamSynchronize(j->stream));
    if (exc(j) && j->d.pxs) {
        // the sums with every walker's waiting measurements folded in, through a
        // scratch of at most 32 MB (whole walkers)
        const size_t per = size_t(2) * j->ch.Nexc * j->ch.Nexc;
        const int chunk = int(std::max<size_t>(1, std::min<size_t>(j->W, (size_t(32) << 20) / (per * sizeof(cx<double>)))));
        void* p = nullptr;
        gv_status st = diag_scratch(j, size_t(chunk) * per * sizeof(cx<double>), &p);
        if (st != GV_OK) return st;
        for (int w0 = 0; w0 < j->W; w0 += chunk) {
            const int nw = std::min(chunk, j->W - w0);
            k_ho_read<256><<<nw, 256, 0, j->stream>>>(j->d, w0, static_cast<cx<double>*>(p));
            GV_CK(cudaGetLastError());
            ++j->total_launches;
            GV_CK(cudaStreamSynchronize(j->stream));
            GV_CK(copy_sync(vals + 2 * per * size_t(w0), p, size_t(nw) * per * sizeof(cx<double>),
                            cudaMemcpyDeviceToHost));
        }
    } else if (exc(j))
        GV_CK(copy_sync(vals, j->d.pjx, sizeof(cx<double>) * 2 * size_t(j->W) * j->ch.Nexc * j->ch.Nexc,
                         cudaMemcpyDeviceToHost));
    else
        GV_CK(copy_sync(vals, j->d.pj, sizeof(cx<double>) * 2 * j->W, cudaMemcpyDeviceToHost));
    if (nmeas) GV_CK(copy_sync(nmeas, j->d.pj_n, sizeof(int32_t) * j->W, cudaMemcpyDeviceToHost));
    return GV_OK;
}

gv_status gv_job_read_orbitals(gv_job* j, int32_t walker, int32_t fl, int32_t* orb)
{
    if (!j || !orb || walker < 0 || walker >= j->W || fl < 0 || fl > 1) return GV_ERR_INVALID;
    if (!exc(j)) {
        for (int f = 0; f < j->N[fl]; ++f) orb[f] = 2 * f;
        return GV_OK;
    }
    GV_CK(cudaStreamSynchronize(j->stream));
    std::vector<int16_t> o(j->Nmax);
    GV_CK(copy_sync(o.data(), j->d.worb + (size_t(walker) * 2 + fl) * j->Nmax, sizeof(int16_t) * j->Nmax,
                     cudaMemcpyDeviceToHost));
    for (int f = 0; f < j->N[fl]; ++f) orb[f] = o[f];
    return GV_OK;
}

gv_status gv_job_read_status(gv_job* j, int32_t* status)
{
    if (!j || !status) return GV_ERR_INVALID;
    GV_CK(cudaStreamSynchronize(j->stream));
    GV_CK(copy_sync(status, j->d.status, sizeof(int32_t) * j->W, cudaMemcpyDeviceToHost));
    return GV_OK;
}

gv_status gv_job_read_weight(gv_job* j, double* sigma)
{
    if (!j || !sigma) return GV_ERR_INVALID;
    if (!exc(j)) {
        for (int w = 0; w < j->W; ++w) sigma[w] = 1.0;
        return GV_OK;
    }
    GV_CK(cudaStreamSynchronize(j->stream));
    GV_CK(copy_sync(sigma, j->d.sigma, sizeof(double) * j->W, cudaMemcpyDeviceToHost));
    return GV_OK;
}

gv_status gv_job_read_stagmagn(gv_job* j, double* vals, int32_t* nmeas)
{
    if (!j || !vals) return GV_ERR_INVALID;
    GV_CK(cudaStreamSynchronize(j->stream));
    GV_CK(copy_sync(vals, j->d.sm, sizeof(cx<double>) * j->W, cudaMemcpyDeviceToHost));
    if (nmeas) GV_CK(copy_sync(nmeas, j->d.sm_n, sizeof(int32_t) * j->W, cudaMemcpyDeviceToHost));
    return GV_OK;
}

// StatSpinStruct m_vals from the compact device sums: with M the number of
// (walker, measurement) pairs, u_i / d_i the times site i held flavour 0 / 1,
//   szz[i][j] = (M - 2 (Aud[i][j] + Aud[j][i])) / 4  (i != j),  szz[i][i] = M / 4
//   s+-[i][j] = -T[j][i] + [i == j] u_i,   s-+[i][j] = -T[i][j] + [i == j] d_i
// (every site is held by exactly one flavour: u_i N_1 = sum_j Aud[i][j],
// d_i N_0 = sum_j Aud[j][i], u_i + d_i = M).
gv_status gv_job_read_statspin(gv_job* j, double* vals, int32_t* nmeas)
{
    if (!j || !vals) return GV_ERR_INVALID;
    GV_CK(cudaStreamSynchronize(j->stream));
    const size_t Ns = size_t(j->Ns), n2 = Ns * Ns;
    std::vector<double> raw(3 * n2);
    GV_CK(copy_sync(raw.data(), j->d.ss, sizeof(double) * 3 * n2, cudaMemcpyDeviceToHost));
    if (nmeas) GV_CK(copy_sync(nmeas, j->d.ss_n, sizeof(int32_t), cudaMemcpyDeviceToHost));
    const double* T = raw.data();
    const double* Aud = raw.data() + 2 * n2;
    std::vector<double> u(Ns, 0.0), dn(Ns, 0.0);
    for (size_t i = 0; i < Ns; ++i)
        for (size_t k = 0; k < Ns; ++k) { u[i] += Aud[i * Ns + k]; dn[i] += Aud[k * Ns + i]; }
    for (size_t i = 0; i < Ns; ++i) { u[i] /= double(j->N[1]); dn[i] /= double(j->N[0]); }
    const double M = Ns ? u[0] + dn[0] : 0.0;
    std::fill(vals, vals + 10 * n2, 0.0);
    double* szz = vals;
    double* spm = vals + 2 * n2;
    double* smp = vals + 4 * n2;
    for (size_t i = 0; i < Ns; ++i)
        for (size_t k = 0; k < Ns; ++k) {
            const size_t ik = i * Ns + k, ki = k * Ns + i;
            szz[2 * ik] = i == k ? 0.25 * M : 0.25 * (M - 2.0 * (Aud[ik] + Aud[ki]));
            spm[2 * ik] = -T[2 * ki] + (i == k ? u[i] : 0.0);
            spm[2 * ik + 1] = -T[2 * ki + 1];
            smp[2 * ik] = -T[2 * ik] + (i == k ? dn[i] : 0.0);
            smp[2 * ik + 1] = -T[2 * ik + 1];
        }
    return GV_OK;
}

// ---- Autotuner: the walk-kernel variants that compute the same chain for a
// job's configuration, timed on a scratch job of the same configuration; the
// fastest is applied to the job and remembered per configuration shape.
namespace {

struct TuneKey {
    int dev, L, channel, precision, flags, wlog;
    bool operator<(const TuneKey& o) const
    {
        return std::tie(dev, L, channel, precision, flags, wlog) <
               std::tie(o.dev, o.L, o.channel, o.precision, o.flags, o.wlog);
    }
};
std::mutex g_tune_mu;
std::map<TuneKey, int> g_tune_cache;

constexpr int kTuneVariants = 5;
constexpr int kTunable = GV_FLAG_DELAYED_UPDATES | GV_FLAG_STREAM_INVERSES;

// Variant v: 0 streaming, default CTA width, immediate updates; 1 the same
// at 256 threads; 2 / 3 as 0 / 1 with delayed updates; 4 on-chip (TMEM).
bool tune_applicable(const gv_job* j, int v)
{
    if (exc(j)) return false;
    const int dflt = pick_threads(j->Nmax);
    const int nt = (v == 1 || v == 3) ? 256 : dflt;
    if ((v == 1 || v == 3) && dflt == 256) return false;   // same as 0 / 2
    if ((v == 2 || v == 3) && j->Nmax > nt) return false;
    if (v == 4) {
        const int f = j->cfg.flags;
        return j->cfg.precision == GV_PREC_MIXED && j->N[0] == j->N[1] && j->Nmax <= 128 &&
               (f & GV_FLAG_REINV_DEFERRED);
    }
    return true;
}

void tune_apply(gv_job* j, int v)
{
    int f = j->cfg.flags & ~kTunable;
    if (v == 2 || v == 3) f |= GV_FLAG_DELAYED_UPDATES;
    if (v != 4 && j->cfg.precision == GV_PREC_MIXED) f |= GV_FLAG_STREAM_INVERSES;
    j->cfg.flags = f;
    j->nt = (v == 1 || v == 3) ? 256 : pick_threads(j->Nmax);
}

}  // namespace

gv_status gv_job_autotune(gv_job* j, uint64_t steps, int32_t* choice, double* us_per_step)
{
    if (!j) return GV_ERR_INVALID;
    if (us_per_step)
        for (int v = 0; v < kTuneVariants; ++v) us_per_step[v] = -1.0;
    if (choice) *choice = -1;
    if (exc(j)) return GV_OK;   // one exciton walk kernel per channel: nothing to choose
    int dev = 0;
    GV_CK(cudaGetDevice(&dev));
    int wlog = 0;
    while ((1 << wlog) < j->W) ++wlog;
    const TuneKey key{dev, j->cfg.L, j->cfg.channel, j->cfg.precision, j->cfg.flags & ~(kTunable | GV_FLAG_CUDA_GRAPHS),
                      wlog};
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {
            tune_apply(j, it->second);
            if (choice) *choice = it->second;
            return GV_OK;
        }
    }
    if (!steps) steps = uint64_t(j->Ns);
    gv_job_config c = j->cfg;
    c.n_walkers = std::min(j->W, 4 * j->n_sm);
    c.meas_mask = 0;
    c.flags &= ~GV_FLAG_CUDA_GRAPHS;
    int best = -1;
    double best_us = 0.0;
    for (int v = 0; v < kTuneVariants; ++v) {
        if (!tune_applicable(j, v)) continue;
        gv_job* s = nullptr;
        gv_status st = gv_job_create(&c, &s);
        if (st) return st;
        tune_apply(s, v);
        double ms = 0.0, tot = 0.0;
        int64_t n = 0;
        if (!(st = gv_job_init_walkers(s, nullptr)) && !(st = gv_job_walk(s, steps, 0)) &&
            !(st = gv_job_synchronize(s)) && !(st = gv_job_timer_start(s)) && !(st = gv_job_walk(s, steps, 0)) &&
            !(st = gv_job_timer_stop(s, &tot, &n)))
            st = gv_job_kernel_ms(s, 0, &ms, &n);   // walk kernels only: the re-inversions are the same for all
        if (!st) st = gv_job_synchronize(s);
        gv_job_destroy(s);
        if (st) return st;
        const double us = ms * 1e3 / double(steps);   // per step of every scratch walker
        if (us_per_step) us_per_step[v] = us;
        if (best < 0 || us < best_us) { best = v; best_us = us; }
    }
    if (best < 0) return GV_OK;
    tune_apply(j, best);
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune_cache[key] = best;
    }
    if (choice) *choice = best;
    return GV_OK;
}

gv_status gv_job_set_track_capacity(gv_job* j, int32_t capacity)
{
    if (!j || capacity < 0) return GV_ERR_INVALID;
    GV_CK(cudaStreamSynchronize(j->stream));
    for (auto& kv : j->graphs) cudaGraphExecDestroy(kv.second.exec);   // they hold the old buffers
    j->graphs.clear();
    cudaFree(j->d.track_sm);
    cudaFree(j->d.track_lw);
    cudaFree(j->d.track_n);
    j->d.track_sm = j->d.track_lw = nullptr;
    j->d.track_n = nullptr;
    j->d.track_cap = 0;
    if (!capacity) return GV_OK;
    const size_t n = size_t(j->W) * capacity;
    if (cudaMalloc(&j->d.track_sm, n * sizeof(double)) || cudaMalloc(&j->d.track_lw, n * sizeof(double)) ||
        cudaMalloc(&j->d.track_n, sizeof(int32_t) * j->W)) {
        cudaGetLastError();
        cudaFree(j->d.track_sm);
        cudaFree(j->d.track_lw);
        cudaFree(j->d.track_n);
        j->d.track_sm = j->d.track_lw = nullptr;
        j->d.track_n = nullptr;
        return GV_ERR_OOM;
    }
    GV_CK(cudaMemset(j->d.track_n, 0, sizeof(int32_t) * j->W));
    j->d.track_cap = capacity;
    return GV_OK;
}

gv_status gv_job_read_tracks(gv_job* j, double* stagmagn, double* log10_weight, int32_t* n)
{
    if (!j) return GV_ERR_INVALID;
    GV_CK(cudaStreamSynchronize(j->stream));
    const size_t m = size_t(j->W) * j->d.track_cap;
    if (!j->d.track_cap) {
        if (n)
            for (int w = 0; w < j->W; ++w) n[w] = 0;
        return GV_OK;
    }
    if (stagmagn) GV_CK(copy_sync(stagmagn, j->d.track_sm, m * sizeof(double), cudaMemcpyDeviceToHost));
    if (log10_weight) GV_CK(copy_sync(log10_weight, j->d.track_lw, m * sizeof(double), cudaMemcpyDeviceToHost));
    if (n) GV_CK(copy_sync(n, j->d.track_n, sizeof(int32_t) * j->W, cudaMemcpyDeviceToHost));
    return GV_OK;
}

gv_status gv_job_graph_stats(gv_job* j, int32_t* cached, int64_t* replays)
{
    if (!j) return GV_ERR_INVALID;
    if (cached) *cached = j->graphs_off ? -1 : int32_t(j->graphs.size());
    if (replays) *replays = j->graph_replays;
    return GV_OK;
}

gv_status gv_job_checkpoint_size(gv_job* j, int32_t flags, uint64_t* bytes)
{
    if (!j || !bytes || (flags & ~GV_CKPT_INVERSES)) return GV_ERR_INVALID;
    uint64_t n = sizeof(CkptHeader);
    for (const CkptSection& s : ckpt_sections(j, flags & GV_CKPT_INVERSES)) n += s.bytes;
    *bytes = n;
    return GV_OK;
}

gv_status gv_job_checkpoint(gv_job* j, int32_t flags, void* buf, uint64_t capacity, uint64_t* written)
{
    uint64_t need = 0;
    if (!buf || gv_job_checkpoint_size(j, flags, &need) || capacity < need) return GV_ERR_INVALID;
    if (!j->ready) return GV_ERR_NOT_READY;
    unsigned char* out = static_cast<unsigned char*>(buf);
    unsigned char* p = out + sizeof(CkptHeader);
    for (const CkptSection& s : ckpt_sections(j, flags & GV_CKPT_INVERSES)) {
        GV_CK(copy_async(p, s.dev, s.bytes, cudaMemcpyDeviceToHost, j->stream));
        p += s.bytes;
    }
    GV_CK(cudaStreamSynchronize(j->stream));
    CkptHeader h = ckpt_header(j, flags);
    h.payload_bytes = uint64_t(p - out) - sizeof(CkptHeader);
    h.checksum = fnv1a64(out + sizeof(CkptHeader), h.payload_bytes);
    std::memcpy(out, &h, sizeof(h));
    if (written) *written = need;
    return GV_OK;
}

gv_status gv_job_restore(gv_job* j, const void* buf, uint64_t size)
{
    if (!j || !buf || size < sizeof(CkptHeader)) return GV_ERR_INVALID;
    CkptHeader h;
    std::memcpy(&h, buf, sizeof(h));
    if (std::memcmp(h.magic, kCkptMagic, sizeof(h.magic)) || h.header_bytes != sizeof(CkptHeader) ||
        (h.flags & ~GV_CKPT_INVERSES) || !ckpt_compatible(h, ckpt_header(j, 0)))
        return GV_ERR_INVALID;
    const bool inverses = (h.flags & GV_CKPT_INVERSES) != 0;
    const std::vector<CkptSection> secs = ckpt_sections(j, inverses);
    uint64_t payload = 0;
    for (const CkptSection& s : secs) payload += s.bytes;
    const unsigned char* in = static_cast<const unsigned char*>(buf) + sizeof(CkptHeader);
    if (h.payload_bytes != payload || size != sizeof(CkptHeader) + payload || fnv1a64(in, payload) != h.checksum)
        return GV_ERR_INVALID;
    GV_CK(cudaStreamSynchronize(j->stream));
    for (const CkptSection& s : secs) {
        GV_CK(copy_async(s.dev, in, s.bytes, cudaMemcpyHostToDevice, j->stream));
        in += s.bytes;
    }
    // The pageable source must outlive the copies: wait before returning.
    GV_CK(cudaStreamSynchronize(j->stream));
    j->ready = true;
    if (inverses) return GV_OK;
    // SlaterDeterminant::Init from the restored configurations (and, for the
    // exciton channel, the overlap rows of the restored channel state).
    gv_status st = invert_all(j);
    if (st) return st;
    GV_CK(cudaMemsetAsync(j->d.since_reinv, 0, sizeof(int32_t) * j->W, j->stream));
    return gv_job_synchronize(j);
}

}  // extern "C"
