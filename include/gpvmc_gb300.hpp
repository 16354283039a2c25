// gpvmc_gb300.hpp -- header-only C++ adapter over the C ABI in gpvmc_gb300.h,
// keeping the reference's class names, signatures and call semantics so that
// a vmc.cpp-style driver, or code that drives the step-level API itself,
// swaps in with few edits:
//
//   reference (EPFL-LQM/gpvmc)                   here
//   BigDouble / BigComplex (BigDouble.h:11,       gv::BigDouble / gv::BigComplex
//     BigComplex.h:10)
//   hop_t / hop_path_t (defs.h:5-7)               gv::hop_t / gv::hop_path_t
//   StagFluxGroundState, StagFluxTransExciton,    gv::StagFluxGroundState, gv::StagFluxTransExciton,
//     StagFluxLongExciton                         gv::StagFluxLongExciton
//     (StagFluxGroundState.cpp:3-15,              GetHops / GetHop from the walker's current state
//      StagFluxTransExciton.cpp:7-44,
//      StagFluxLongExciton.cpp:6-66;
//      WaveFunction.cpp:69-83)
//   SlaterDeterminant (SlaterDeterminant.h:44)    gv::SlaterDeterminant  Init, Amp, VirtUpdate(rhop, khop, qs),
//                                                                        Update(rhop, khop)
//   Stepper / LatticeStepper (Stepper.h:13-34,    gv::LatticeStepper     Reset, trystep, step, weight, transprob,
//     LatticeStepper.h:16)                                               GetAmp, GetWaveFunction
//   MetroMC (MetroMC.h:11)                        gv::MetroMC            AddQuantity, Walk, Step, YesNo, Rejection
//   ProjHeis / StagMagnZ / StatSpinStruct         gv::ProjHeis / gv::StagMagnZ / gv::StatSpinStruct
//     (ProjHeis.h, StagMagnZ.h, StatSpinStruct.h)  init, save, GetNmeas
//
// One gv::Job holds n_walkers independent chains (the reference: one chain
// per MPI rank); the step-level objects act on one walker of it (default 0).
// MetroMC::Walk runs every walker of the job on the GPU at once; MetroMC::Step
// steps one walker through the single-walker entry points (same Philox
// stream, same update kernels).  Errors throw gv::Error (the reference throws
// std::logic_error under -DEXCEPT and aborts otherwise).
#pragma once

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "gpvmc_gb300.h"

namespace gv {

class Error : public std::runtime_error {
  public:
    Error(gv_status s, const char* where)
        : std::runtime_error(std::string(where) + ": " + gv_status_string(s)), status(s) {}
    gv_status status;
};

inline void check(gv_status s, const char* where)
{
    if (s != GV_OK) throw Error(s, where);
}

// A positive real with an integer exponent, m * 2^e with m in [0.5, 1) (or
// 0): the weights of the reference's BigDouble (base 10 there; base 2 here,
// so that renormalising is exact).  The operations the hot path uses: *, /,
// comparison, conversion to double.
class BigDouble {
  public:
    BigDouble(double v = 0.0) { set(v, 0); }
    BigDouble(double m, int e2) { set(m, e2); }
    double mantissa() const { return m_; }
    int exponent2() const { return e_; }
    operator double() const { return std::ldexp(m_, e_); }
    double log10() const { return m_ > 0 ? std::log10(m_) + e_ * 0.30102999566398119521 : -HUGE_VAL; }
    friend BigDouble operator*(const BigDouble& a, const BigDouble& b) { return BigDouble(a.m_ * b.m_, a.e_ + b.e_); }
    friend BigDouble operator/(const BigDouble& a, const BigDouble& b) { return BigDouble(a.m_ / b.m_, a.e_ - b.e_); }
    friend bool operator<(const BigDouble& a, const BigDouble& b)
    {
        if (a.m_ == 0 || b.m_ == 0) return a.m_ < b.m_;
        return a.e_ < b.e_ || (a.e_ == b.e_ && a.m_ < b.m_);
    }
    friend bool operator>(const BigDouble& a, const BigDouble& b) { return b < a; }

  private:
    void set(double m, int e2)
    {
        int k = 0;
        m_ = std::frexp(m, &k);
        e_ = m_ == 0.0 ? 0 : e2 + k;
    }
    double m_ = 0.0;
    int e_ = 0;
};

// A complex value as the reference's BigComplex: mantissa with |m| in [1, 10)
// (or 0) and a base-10 exponent (BigComplex.h:16-44).
class BigComplex {
  public:
    BigComplex(std::complex<double> v = 0.0) { set(v, 0); }
    BigComplex(std::complex<double> m, int e10) { set(m, e10); }
    std::complex<double> mantissa() const { return m_; }
    int exponent10() const { return e_; }
    // value (may overflow for large lattices: compare mantissa and exponent instead)
    std::complex<double> value() const { return m_ * std::pow(10.0, e_); }
    friend BigComplex operator*(const BigComplex& a, std::complex<double> b) { return BigComplex(a.m_ * b, a.e_); }
    friend BigDouble norm(const BigComplex& a)
    {
        // |m|^2 10^(2e) as mantissa * 2^e2
        const double l2 = 2.0 * a.e_ * 3.32192809488736234787;
        const double fl = std::floor(l2);
        return BigDouble(std::norm(a.m_) * std::exp2(l2 - fl), int(fl));
    }

  private:
    void set(std::complex<double> m, int e10)
    {
        const double a = std::abs(m);
        if (a == 0.0) { m_ = 0.0; e_ = 0; return; }
        int k = int(std::floor(std::log10(a)));
        m_ = m / std::pow(10.0, k);
        e_ = e10 + k;
        if (std::abs(m_) >= 10.0) { m_ /= 10.0; ++e_; }
        if (std::abs(m_) < 1.0) { m_ *= 10.0; --e_; }
    }
    std::complex<double> m_ = 0.0;
    int e_ = 0;
};

// hop_t: (from, to) fock index -- a lattice site for the real-space hops of
// these channels (one internal state per site and flavour), an orbital for
// the wavefunction's hops; hop_path_t: the hops of one flavour (defs.h:5-7).
typedef std::pair<size_t, size_t> hop_t;
typedef std::vector<hop_t> hop_path_t;

// StagFluxWaveFunction parameters (StagFluxWaveFunction.cpp:8-43); phi in
// radians as the reference's constructor receives it.
struct WaveFunctionParams {
    int L;
    int channel;
    int q[2];
    double phi, neel, neel_exp;
    double phase_shift[2];
};

struct StagFluxGroundState : WaveFunctionParams {
    StagFluxGroundState(int L_, double phi_, double neel_, double neel_exp_ = 0.0, double bcx = 1.0, double bcy = 1.0)
        : WaveFunctionParams{L_, GV_CH_GROUNDSTATE, {0, 0}, phi_, neel_, neel_exp_, {bcx, bcy}} {}
};

// StagFluxTransExciton (StagFluxTransExciton.cpp:7-44): momentum q = (qx, qy).
struct StagFluxTransExciton : WaveFunctionParams {
    StagFluxTransExciton(int L_, double phi_, double neel_, int qx, int qy, double neel_exp_ = 0.0, double bcx = 1.0,
                         double bcy = 1.0)
        : WaveFunctionParams{L_, GV_CH_TRANS, {qx, qy}, phi_, neel_, neel_exp_, {bcx, bcy}} {}
};

// StagFluxLongExciton (StagFluxLongExciton.cpp:6-66): momentum q = (qx, qy);
// L^2 particle-hole states within one flavour plus the unexcited state.
struct StagFluxLongExciton : WaveFunctionParams {
    StagFluxLongExciton(int L_, double phi_, double neel_, int qx, int qy, double neel_exp_ = 0.0, double bcx = 1.0,
                        double bcy = 1.0)
        : WaveFunctionParams{L_, GV_CH_LONG, {qx, qy}, phi_, neel_, neel_exp_, {bcx, bcy}} {}
};

class Job {
  public:
    Job(const WaveFunctionParams& wav, int n_walkers, uint64_t seed, int precision = GV_PREC_FP64,
        int reinv_every = 0, int flags = 0, double drift_threshold = 0.0)
        : wav_(wav)
    {
        gv_job_config c = {};
        c.L = wav.L;
        c.channel = wav.channel;
        c.q[0] = wav.q[0];
        c.q[1] = wav.q[1];
        c.phi = wav.phi;
        c.neel = wav.neel;
        c.neel_exp = wav.neel_exp;
        c.phase_shift[0] = wav.phase_shift[0];
        c.phase_shift[1] = wav.phase_shift[1];
        c.n_walkers = n_walkers;
        c.precision = precision;
        c.seed = seed;
        c.reinv_every = reinv_every;
        c.flags = flags;
        c.drift_threshold = drift_threshold;
        check(gv_job_create(&c, &job_), "gv_job_create");
        check(gv_job_dims(job_, &Ns_, &N_[0], &N_[1], &Nexc_), "gv_job_dims");
        walkers_ = n_walkers;
        if (wav.channel != GV_CH_GROUNDSTATE) {
            exc_up_.resize(Nexc_);
            exc_dn_.resize(Nexc_);
            check(gv_channel_states(wav.L, wav.phase_shift, wav.channel, wav.q, exc_up_.data(), exc_dn_.data()),
                  "gv_channel_states");
        }
    }
    ~Job() { gv_job_destroy(job_); }
    Job(const Job&) = delete;
    Job& operator=(const Job&) = delete;

    gv_job* handle() const { return job_; }
    int walkers() const { return walkers_; }
    int Ns() const { return Ns_; }
    int Nexc() const { return Nexc_; }
    int N(int fl) const { return N_[fl]; }
    const WaveFunctionParams& wav() const { return wav_; }
    const std::vector<int32_t>& exc_up() const { return exc_up_; }
    const std::vector<int32_t>& exc_dn() const { return exc_dn_; }
    // LatticeState::RanInit / FockInit + SlaterDeterminant::Init (vmc.cpp:161-263)
    void InitWalkers(const std::vector<int8_t>* up = nullptr)
    {
        check(gv_job_init_walkers(job_, up ? up->data() : nullptr), "gv_job_init_walkers");
    }
    void SetMeasurements(int mask) { check(gv_job_set_meas_mask(job_, mask), "gv_job_set_meas_mask"); }
    void Walk(uint64_t len, uint64_t meas)
    {
        check(gv_job_walk(job_, len, meas), "gv_job_walk");
        check(gv_job_synchronize(job_), "gv_job_synchronize");
    }
    // Quantity::measure of the attached quantities on the current configurations
    void Measure() { check(gv_job_measure(job_), "gv_job_measure"); }
    // LatticeState::Getfs: 1 where flavour 0 sits, per site, of one walker
    std::vector<int8_t> Config(int walker = 0) const
    {
        std::vector<int8_t> all(size_t(walkers_) * Ns_);
        check(gv_job_read_config(job_, all.data()), "gv_job_read_config");
        return std::vector<int8_t>(all.begin() + size_t(walker) * Ns_, all.begin() + size_t(walker + 1) * Ns_);
    }
    // WaveFunction::m_c_exc of one walker
    int CurrentState(int walker = 0) const
    {
        std::vector<int32_t> s(walkers_);
        check(gv_job_read_state_index(job_, s.data()), "gv_job_read_state_index");
        return s[walker];
    }
    // State::Save (State.cpp:117-166) with the Philox counters, counters and
    // quantity sums; with inverses the restored chain continues bit for bit.
    std::vector<unsigned char> Checkpoint(bool inverses = false)
    {
        const int32_t fl = inverses ? GV_CKPT_INVERSES : 0;
        uint64_t n = 0;
        check(gv_job_checkpoint_size(job_, fl, &n), "gv_job_checkpoint_size");
        std::vector<unsigned char> blob(n);
        check(gv_job_checkpoint(job_, fl, blob.data(), n, nullptr), "gv_job_checkpoint");
        return blob;
    }
    // The --spinstate resume (vmc.cpp:178-220) from a blob of a job with the same configuration.
    void Restore(const std::vector<unsigned char>& blob)
    {
        check(gv_job_restore(job_, blob.data(), blob.size()), "gv_job_restore");
    }

  private:
    gv_job* job_ = nullptr;
    WaveFunctionParams wav_;
    int32_t Ns_ = 0, N_[2] = {0, 0}, Nexc_ = 0;
    int walkers_ = 0;
    std::vector<int32_t> exc_up_, exc_dn_;
};

// The wavefunction of one walker: its channel states and the hops between
// them (WaveFunction::GetHops / GetHop, WaveFunction.cpp:69-83); the ground
// state has one state and no hops.  Transverse exciton: from the current
// state c, state k differs by flavour 0: exc_up[c] -> exc_up[k] and flavour 1:
// exc_dn[k] -> exc_dn[c] (none for k = c).  Longitudinal exciton: state
// k < Ns lifts one particle of flavour k % 2 from orbital exc_dn[k] to
// exc_up[k], state Ns lifts none; from c to k a flavour carrying both
// excitations takes the two hops {exc_up[c], exc_dn[k]} -> {exc_up[k],
// exc_dn[c]} (each side in increasing order, paired in that order), one
// carrying only c's undoes it (exc_up[c] -> exc_dn[c]), one carrying only k's
// makes it (exc_dn[k] -> exc_up[k]).
class WaveFunction {
  public:
    WaveFunction(Job& job, int walker = 0) : job_(job), walker_(walker) {}
    int GetNExc() const { return job_.Nexc(); }
    int GetCurrentState() const { return job_.wav().channel != GV_CH_GROUNDSTATE ? job_.CurrentState(walker_) : 0; }
    std::vector<std::vector<hop_path_t>> GetHops() const
    {
        const int Nexc = job_.Nexc();
        std::vector<std::vector<hop_path_t>> h(Nexc, std::vector<hop_path_t>(2));
        if (job_.wav().channel == GV_CH_GROUNDSTATE) return h;
        const int c = GetCurrentState();
        const std::vector<int32_t>& up = job_.exc_up();
        const std::vector<int32_t>& dn = job_.exc_dn();
        if (job_.wav().channel == GV_CH_TRANS) {
            for (int k = 0; k < Nexc; ++k) {
                if (k == c) continue;
                h[k][0].push_back(hop_t(up[c], up[k]));
                h[k][1].push_back(hop_t(dn[k], dn[c]));
            }
            return h;
        }
        const int Ns = job_.Ns();
        auto kind = [Ns](int k) { return k < Ns ? (k & 1) : 2; };
        for (int k = 0; k < Nexc; ++k)
            for (int fl = 0; fl < 2; ++fl) {
                const bool ec = kind(c) == fl, ek = kind(k) == fl;
                if (ec && ek && k != c) {
                    const std::pair<int, int> v = std::minmax(up[c], dn[k]), f = std::minmax(up[k], dn[c]);
                    h[k][fl].push_back(hop_t(v.first, f.first));
                    h[k][fl].push_back(hop_t(v.second, f.second));
                } else if (ec && !ek) {
                    h[k][fl].push_back(hop_t(up[c], dn[c]));
                } else if (ek && !ec) {
                    h[k][fl].push_back(hop_t(dn[k], up[k]));
                }
            }
        return h;
    }
    std::vector<hop_path_t> GetHop(int k) const { return GetHops()[k]; }
    // index of the state a hop set leads to from the current state, -1 if none
    int StateOf(const std::vector<hop_path_t>& khop) const
    {
        const auto h = GetHops();
        for (size_t k = 0; k < h.size(); ++k)
            if (khop.size() == 2 && h[k][0] == khop[0] && h[k][1] == khop[1]) return int(k);
        return -1;
    }
    Job& job() const { return job_; }
    int walker() const { return walker_; }

  private:
    Job& job_;
    int walker_;
};

class SlaterDeterminant {
  public:
    explicit SlaterDeterminant(Job& job, int walker = 0) : job_(job), walker_(walker) {}
    // SlaterDeterminant::Init on every walker of the job (FP64 LU re-inversion)
    void Init() { check(gv_job_reinvert(job_.handle()), "gv_job_reinvert"); }
    // Amp() of one walker as a complex value (may overflow for large L: use AmpParts / BigAmp)
    std::complex<double> Amp(int walker) const
    {
        double m[2];
        int32_t e;
        AmpParts(walker, m, &e);
        return std::complex<double>(m[0], m[1]) * std::pow(10.0, e);
    }
    BigComplex BigAmp(int walker) const
    {
        double m[2];
        int32_t e;
        AmpParts(walker, m, &e);
        return BigComplex(std::complex<double>(m[0], m[1]), e);
    }
    // SlaterDeterminant::Amp (SlaterDeterminant.cpp:94) of this object's walker
    BigComplex Amp() const { return BigAmp(walker_); }
    void AmpParts(int walker, double* mant, int32_t* exp10) const
    {
        std::vector<double> m(2 * job_.walkers());
        std::vector<int32_t> e(job_.walkers());
        check(gv_job_read_amplitude(job_.handle(), m.data(), e.data()), "gv_job_read_amplitude");
        mant[0] = m[2 * walker];
        mant[1] = m[2 * walker + 1];
        *exp10 = e[walker];
    }
    // VirtUpdate ratios qs/Amp() for swap sets (up_from, up_to, dn_from, dn_to), -1 = none
    // (ground state: one value per set; exciton channel: [state][set])
    std::vector<std::complex<double>> VirtUpdate(const std::vector<int32_t>& hops, int walker = 0) const
    {
        const int n = int(hops.size() / 4);
        const int K = job_.Nexc();
        std::vector<double> out(2 * size_t(n) * K);
        check(gv_job_virt_update(job_.handle(), walker, n, hops.data(), out.data()), "gv_job_virt_update");
        std::vector<std::complex<double>> q(size_t(n) * K);
        for (size_t i = 0; i < q.size(); ++i) q[i] = std::complex<double>(out[2 * i], out[2 * i + 1]);
        return q;
    }
    // SlaterDeterminant::VirtUpdate (SlaterDeterminant.h:50-53): for every
    // real-space hop set rhop[r] (per flavour at most one hop: the
    // spin-exchange moves of these channels) and every wavefunction hop set
    // khop[k] (a hop from the current state, as WaveFunction::GetHops gives
    // them), qs[k * rhop.size() + r] = <configuration after rhop[r] | state
    // after khop[k]>, including the wavefunction's hop sign.
    void VirtUpdate(const std::vector<std::vector<hop_path_t>>& rhop, const std::vector<std::vector<hop_path_t>>& khop,
                    std::vector<BigComplex>& qs) const
    {
        const int Nr = int(rhop.size());
        std::vector<int32_t> hops(4 * size_t(Nr), -1);
        for (int r = 0; r < Nr; ++r) {
            if (rhop[r].size() != 2 || rhop[r][0].size() > 1 || rhop[r][1].size() > 1)
                throw Error(GV_ERR_INVALID, "SlaterDeterminant::VirtUpdate: one hop per flavour at most");
            for (int fl = 0; fl < 2; ++fl)
                if (!rhop[r][fl].empty()) {
                    hops[4 * r + 2 * fl] = int32_t(rhop[r][fl][0].first);
                    hops[4 * r + 2 * fl + 1] = int32_t(rhop[r][fl][0].second);
                }
        }
        const WaveFunction wav(job_, walker_);
        std::vector<int> state(khop.size());
        for (size_t k = 0; k < khop.size(); ++k) {
            state[k] = wav.StateOf(khop[k]);
            if (state[k] < 0) throw Error(GV_ERR_INVALID, "SlaterDeterminant::VirtUpdate: not a hop of the wavefunction");
        }
        const auto rel = VirtUpdate(hops, walker_);   // [state][set], relative to Amp()
        const BigComplex a = Amp();
        qs.assign(khop.size() * Nr, BigComplex());
        for (size_t k = 0; k < khop.size(); ++k)
            for (int r = 0; r < Nr; ++r) qs[k * Nr + r] = a * rel[size_t(state[k]) * Nr + r];
    }
    // SlaterDeterminant::Update (SlaterDeterminant.h:55-56) together with the
    // lattice and wavefunction hops it follows in LatticeStepper::step: the
    // exchange rhop (flavour 0 from a to b, flavour 1 from b to a) and the
    // wavefunction hop khop (empty hops: stay in the current state).
    void Update(const std::vector<hop_path_t>& rhop, const std::vector<hop_path_t>& khop)
    {
        int32_t hop[4] = {-1, -1, -1, -1};
        if (rhop.size() != 2 || rhop[0].size() > 1 || rhop[1].size() > 1)
            throw Error(GV_ERR_INVALID, "SlaterDeterminant::Update: one hop per flavour at most");
        for (int fl = 0; fl < 2; ++fl)
            if (!rhop[fl].empty()) {
                hop[2 * fl] = int32_t(rhop[fl][0].first);
                hop[2 * fl + 1] = int32_t(rhop[fl][0].second);
            }
        const int state = WaveFunction(job_, walker_).StateOf(khop);
        if (state < 0) throw Error(GV_ERR_INVALID, "SlaterDeterminant::Update: not a hop of the wavefunction");
        check(gv_job_update(job_.handle(), walker_, hop, state), "gv_job_update");
    }
    int walker() const { return walker_; }

  private:
    Job& job_;
    int walker_;
};

// Stepper (Stepper.h:13-34) / LatticeStepper (LatticeStepper.cpp:36-174) of one walker.
class LatticeStepper {
  public:
    explicit LatticeStepper(Job& job, int walker = 0) : job_(job), walker_(walker), amp_(job, walker), wav_(job, walker) {}
    Job& job() const { return job_; }
    int walker() const { return walker_; }
    void Reset() { khop_ = -1; pending_ = false; }
    // the proposal's weight sum_k |q_k|^2 (the current weight for a same-flavour proposal)
    BigDouble trystep()
    {
        double m = 0.0;
        int32_t e = 0, k = -1;
        check(gv_job_trystep(job_.handle(), walker_, prev_, &m, &e, &k), "gv_job_trystep");
        khop_ = k;
        pending_ = true;
        return BigDouble(m, e);
    }
    void step()
    {
        if (!pending_) throw Error(GV_ERR_INVALID, "LatticeStepper::step: no trystep");
        pending_ = false;
        check(gv_job_step(job_.handle(), walker_), "gv_job_step");
        khop_ = -1;
    }
    BigDouble weight() const
    {
        double m = 0.0;
        int32_t e = 0;
        check(gv_job_stepper_weight(job_.handle(), walker_, &m, &e), "gv_job_stepper_weight");
        return BigDouble(m, e);
    }
    double transprob() const { return 1.0; }
    // the last trystep's vertices and arg-max channel state (-1: same-flavour proposal)
    int Proposal(int i) const { return prev_[i]; }
    int Khop() const { return khop_; }
    const SlaterDeterminant* GetAmp() const { return &amp_; }
    SlaterDeterminant* GetAmp() { return &amp_; }
    const WaveFunction* GetWaveFunction() const { return &wav_; }

  private:
    Job& job_;
    int walker_;
    SlaterDeterminant amp_;
    WaveFunction wav_;
    int32_t prev_[2] = {-1, -1};
    int khop_ = -1;
    bool pending_ = false;
};

class Quantity {
  public:
    explicit Quantity(const LatticeStepper& s, int mask) : job_(s.job()), mask_(mask) {}
    virtual ~Quantity() {}
    int mask() const { return mask_; }
    void init() { check(gv_job_reset_quantities(job_.handle()), "gv_job_reset_quantities"); }

  protected:
    Job& job_;
    int mask_;
};

// ProjHeis (ProjHeis.cpp:40-158), ground state: per walker [E/site sum, count].
class ProjHeis : public Quantity {
  public:
    explicit ProjHeis(const LatticeStepper& s) : Quantity(s, GV_MEAS_PROJHEIS) {}
    // m_vals / m_meas per walker (MatrixQuantity::save, MatrixQuantity.cpp:12-17)
    std::vector<std::complex<double>> save() const
    {
        std::vector<double> v(4 * job_.walkers());
        std::vector<int32_t> n(job_.walkers());
        check(gv_job_read_projheis(job_.handle(), v.data(), n.data()), "gv_job_read_projheis");
        std::vector<std::complex<double>> e(job_.walkers());
        for (int w = 0; w < job_.walkers(); ++w)
            e[w] = std::complex<double>(v[4 * w], v[4 * w + 1]) / double(n[w] ? n[w] : 1);
        return e;
    }
    int GetNmeas(int walker = 0) const
    {
        std::vector<double> v(4 * job_.walkers());
        std::vector<int32_t> n(job_.walkers());
        check(gv_job_read_projheis(job_.handle(), v.data(), n.data()), "gv_job_read_projheis");
        return n[walker];
    }
};

class StagMagnZ : public Quantity {
  public:
    explicit StagMagnZ(const LatticeStepper& s) : Quantity(s, GV_MEAS_STAGMAGN) {}
    std::vector<std::complex<double>> save() const
    {
        std::vector<double> v(2 * job_.walkers());
        std::vector<int32_t> n(job_.walkers());
        check(gv_job_read_stagmagn(job_.handle(), v.data(), n.data()), "gv_job_read_stagmagn");
        std::vector<std::complex<double>> m(job_.walkers());
        for (int w = 0; w < job_.walkers(); ++w)
            m[w] = std::complex<double>(v[2 * w], v[2 * w + 1]) / double(n[w] ? n[w] : 1);
        return m;
    }
};

class StatSpinStruct : public Quantity {
  public:
    explicit StatSpinStruct(const LatticeStepper& s) : Quantity(s, GV_MEAS_STATSPIN) {}
    // 5 x Ns x Ns sums over all walkers divided by the measurements per walker
    std::vector<std::complex<double>> save() const
    {
        const size_t n2 = size_t(job_.Ns()) * job_.Ns();
        std::vector<double> v(10 * n2);
        int32_t n = 0;
        check(gv_job_read_statspin(job_.handle(), v.data(), &n), "gv_job_read_statspin");
        std::vector<std::complex<double>> s(5 * n2);
        for (size_t i = 0; i < 5 * n2; ++i) s[i] = std::complex<double>(v[2 * i], v[2 * i + 1]) / double(n ? n : 1);
        return s;
    }
};

class MetroMC {
  public:
    explicit MetroMC(LatticeStepper& s) : job_(s.job()), stepper_(s) {}
    void AddQuantity(Quantity* q)
    {
        mask_ |= q->mask();
        check(gv_job_set_meas_mask(job_.handle(), mask_), "gv_job_set_meas_mask");
    }
    // MetroMC::Walk (MetroMC.cpp:45-88) on every walker of the job at once
    void Walk(uint64_t len, uint64_t meas)
    {
        job_.Walk(len, meas);
        have_weight_ = false;   // the walk moved the stepper's walker too
    }
    // MetroMC::Step (MetroMC.cpp:90-103) of the stepper's walker
    void Step(bool meas)
    {
        if (!have_weight_) {   // the weight of the current state (MetroMC ctor, MetroMC.cpp:24)
            state_weight_ = stepper_.weight();
            have_weight_ = true;
        }
        const BigDouble new_weight = stepper_.trystep();
        if (YesNo(new_weight / state_weight_)) {
            stepper_.step();
            state_weight_ = new_weight;
        } else if (meas) {
            ++rejection_;
        }
        if (meas) ++steps_;
    }
    // MetroMC::YesNo (MetroMC.cpp:27-43): the step's u4 against min(1, in)
    bool YesNo(const BigDouble& in)
    {
        int32_t acc = 0;
        check(gv_job_yesno(job_.handle(), stepper_.walker(), double(in), &acc), "gv_job_yesno");
        return acc != 0;
    }
    // MetroMC::Rejection (MetroMC.cpp:105-111) of one walker, over all its steps
    double Rejection(int walker = 0) const
    {
        std::vector<uint64_t> c(5 * job_.walkers());
        check(gv_job_read_counts(job_.handle(), c.data()), "gv_job_read_counts");
        const uint64_t steps = c[5 * walker];
        return steps ? double(c[5 * walker + 3]) / double(steps) : 0.0;
    }
    // over the measured Step calls only, as the reference counts them
    double StepRejection() const { return steps_ ? double(rejection_) / double(steps_) : 0.0; }

  private:
    Job& job_;
    LatticeStepper& stepper_;
    int mask_ = 0;
    BigDouble state_weight_;
    bool have_weight_ = false;
    uint64_t steps_ = 0, rejection_ = 0;
};

}  // namespace gv
