// gpvmc_gb300.hpp -- header-only C++ adapter over the C ABI in gpvmc_gb300.h,
// keeping the reference's class names and call semantics so that a
// vmc.cpp-style driver swaps in with few edits:
//
//   reference (EPFL-LQM/gpvmc)                  here
//   SlaterDeterminant (SlaterDeterminant.h:44)  gv::SlaterDeterminant  Init, Amp, VirtUpdate
//   LatticeStepper (LatticeStepper.h:16)        gv::LatticeStepper
//   MetroMC (MetroMC.h:11)                      gv::MetroMC            AddQuantity, Walk, Rejection
//   ProjHeis / StagMagnZ / StatSpinStruct       gv::ProjHeis / gv::StagMagnZ / gv::StatSpinStruct
//   (ProjHeis.h, StagMagnZ.h, StatSpinStruct.h) init, save, GetNmeas
//
// One gv::Job holds n_walkers independent chains (the reference: one chain
// per MPI rank).  Errors throw gv::Error (the reference throws
// std::logic_error under -DEXCEPT and aborts otherwise).
#pragma once

#include <complex>
#include <cstdint>
#include <stdexcept>
#include <string>
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

// StagFluxWaveFunction parameters (StagFluxWaveFunction.cpp:8-43); phi in
// radians as the reference's constructor receives it.
struct StagFluxGroundState {
    int L;
    double phi, neel, neel_exp;
    double phase_shift[2];
    StagFluxGroundState(int L_, double phi_, double neel_, double neel_exp_ = 0.0, double bcx = 1.0, double bcy = 1.0)
        : L(L_), phi(phi_), neel(neel_), neel_exp(neel_exp_), phase_shift{bcx, bcy} {}
};

class Job {
  public:
    Job(const StagFluxGroundState& wav, int n_walkers, uint64_t seed, int precision = GV_PREC_FP64,
        int reinv_every = 0, int flags = 0, double drift_threshold = 0.0)
    {
        gv_job_config c = {};
        c.L = wav.L;
        c.channel = GV_CH_GROUNDSTATE;
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
    }
    ~Job() { gv_job_destroy(job_); }
    Job(const Job&) = delete;
    Job& operator=(const Job&) = delete;

    gv_job* handle() const { return job_; }
    int walkers() const { return walkers_; }
    int Ns() const { return Ns_; }
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
    int32_t Ns_ = 0, N_[2] = {0, 0}, Nexc_ = 0;
    int walkers_ = 0;
};

class SlaterDeterminant {
  public:
    explicit SlaterDeterminant(Job& job) : job_(job) {}
    void Init() { check(gv_job_reinvert(job_.handle()), "gv_job_reinvert"); }
    // Amp() of one walker as a complex value (may overflow for large L: use AmpLog10)
    std::complex<double> Amp(int walker = 0) const
    {
        double m[2];
        int32_t e;
        AmpParts(walker, m, &e);
        return std::complex<double>(m[0], m[1]) * std::pow(10.0, e);
    }
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
    std::vector<std::complex<double>> VirtUpdate(const std::vector<int32_t>& hops, int walker = 0) const
    {
        const int n = int(hops.size() / 4);
        std::vector<double> out(2 * n);
        check(gv_job_virt_update(job_.handle(), walker, n, hops.data(), out.data()), "gv_job_virt_update");
        std::vector<std::complex<double>> q(n);
        for (int i = 0; i < n; ++i) q[i] = std::complex<double>(out[2 * i], out[2 * i + 1]);
        return q;
    }

  private:
    Job& job_;
};

class LatticeStepper {
  public:
    explicit LatticeStepper(Job& job) : job_(job) {}
    Job& job() const { return job_; }

  private:
    Job& job_;
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
    explicit MetroMC(LatticeStepper& s) : job_(s.job()) {}
    void AddQuantity(Quantity* q)
    {
        mask_ |= q->mask();
        check(gv_job_set_meas_mask(job_.handle(), mask_), "gv_job_set_meas_mask");
    }
    void Walk(uint64_t len, uint64_t meas) { job_.Walk(len, meas); }
    // MetroMC::Rejection (MetroMC.cpp:105-111) of one walker
    double Rejection(int walker = 0) const
    {
        std::vector<uint64_t> c(5 * job_.walkers());
        check(gv_job_read_counts(job_.handle(), c.data()), "gv_job_read_counts");
        const uint64_t steps = c[5 * walker];
        return steps ? double(c[5 * walker + 3]) / double(steps) : 0.0;
    }

  private:
    Job& job_;
    int mask_ = 0;
};

}  // namespace gv
