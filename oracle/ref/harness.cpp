// Drives the reference's own classes (compiled unmodified from the reference
// sources by oracle/ref/Makefile) behind the same extern "C" surface as the
// C restatement in oracle/vmc_oracle.h, so that one test script can run both
// and compare.  Test infrastructure only; it reads private/protected state
// of the reference objects (inverse matrices, accumulators) to dump golden
// vectors, which is why the access specifiers are opened below.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <limits>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>
#include <fcntl.h>
#include <unistd.h>

#define private public
#define protected public
#include "BigComplex.h"
#include "BigDouble.h"
#include "FileManager.h"
#include "LatticeState.h"
#include "LatticeStepper.h"
#include "MetroMC.h"
#include "ProjHeis.h"
#include "SlaterDeterminant.h"
#include "SquareLattice.h"
#include "StagFluxGroundState.h"
#include "StagFluxLongExciton.h"
#include "StagFluxTransExciton.h"
#include "StagMagnZ.h"
#include "StatSpinStruct.h"
#include "Stepper.h"
#include "WaveFunction.h"
#undef private
#undef protected

#include "../vmc_oracle.h"

extern "C" void ref_rng_set(uint64_t seed, uint32_t walker, uint32_t stream, uint64_t next);
extern "C" uint64_t ref_rng_next(void);
extern "C" double ref_rng_peek(uint64_t k);

namespace {

// Forwards to the reference LatticeStepper and records whether step() ran.
class TraceStepper : public Stepper {
  public:
    TraceStepper(LatticeState* ls, WaveFunction* wav, SlaterDeterminant* amp)
        : Stepper(ls, wav, amp), inner(ls, wav, amp), stepped(false) {}
    void Reset() override { inner.Reset(); }
    BigDouble trystep() override { return inner.trystep(); }
    void step() override { inner.step(); stepped = true; }
    BigDouble weight() override { return inner.weight(); }
    BigDouble weight() const override { return static_cast<const LatticeStepper&>(inner).weight(); }
    double transprob() override { return inner.transprob(); }
    LatticeStepper inner;
    bool stepped;
};

struct RefRun {
    int L = 0, channel = 0;
    FileManager* fm = nullptr;
    SquareLattice* lat = nullptr;
    LatticeState* sp = nullptr;
    WaveFunction* wav = nullptr;
    SlaterDeterminant* amp = nullptr;
    TraceStepper* step = nullptr;
    MetroMC* mc = nullptr;
    ProjHeis* pj = nullptr;
    StagMagnZ* sm = nullptr;
    StatSpinStruct* ss = nullptr;
    uint64_t seed = 0;
    uint32_t walker = 0;
    uint64_t next = 0;
    uint64_t accepted_real = 0, reinversions = 0, since_reinv = 0;
};

void teardown_chain(RefRun* r)
{
    delete r->pj; delete r->sm; delete r->ss; delete r->mc; delete r->step;
    r->pj = nullptr; r->sm = nullptr; r->ss = nullptr; r->mc = nullptr; r->step = nullptr;
}

// vmc.cpp:243-285: arg-max over channel states, then stepper, MetroMC and
// the quantities.
int finish_start(RefRun* r)
{
    BigDouble maxq = norm(r->amp->Amp());
    size_t kmax = r->wav->GetCurrentStateIndex();
    for (size_t k = 0; k < r->wav->GetNExc(); ++k) {
        r->wav->Hop(k);
        r->amp->Init();
        if (norm(r->amp->Amp()) > maxq) { kmax = k; maxq = norm(r->amp->Amp()); }
    }
    r->wav->Hop(kmax);
    r->amp->Init();
    if (r->amp->Amp() == 0.0) return ORC_ERR_SINGULAR;
    teardown_chain(r);
    r->step = new TraceStepper(r->sp, r->wav, r->amp);
    r->mc = new MetroMC(r->step, r->fm);
    r->pj = new ProjHeis(r->step, r->fm, r->lat, 0.0);
    r->sm = new StagMagnZ(r->step, r->fm);
    r->ss = new StatSpinStruct(r->step, r->fm, true);
    r->next = 0;
    return ORC_OK;
}

void select_quantities(RefRun* r, int mask)
{
    std::vector<Quantity*>& q = r->mc->GetQuantities();
    q.clear();
    if (mask & ORC_MEAS_PROJHEIS) q.push_back(r->pj);
    if (mask & ORC_MEAS_STAGMAGN) q.push_back(r->sm);
    if (mask & ORC_MEAS_STATSPIN) q.push_back(r->ss);
}

int one_step(RefRun* r, int meas, orc_trace* tr)
{
    ref_rng_set(r->seed, r->walker, 0, r->next);
    uint64_t k0 = r->next;
    std::vector<uint_vec_t> before = r->sp->Getfs();
    BigDouble sw = r->mc->m_state_weight;
    r->step->stepped = false;
    try {
        r->mc->Step(meas != 0);
    } catch (std::exception&) {
        return ORC_ERR_SINGULAR;
    }
    r->next = ref_rng_next();
    if (r->next - k0 != 4) return ORC_ERR_INVALID;
    bool real = before != r->sp->Getfs();
    if (r->step->stepped && real) { r->accepted_real++; r->since_reinv++; }
    if (tr) {
        std::memset(tr, 0, sizeof *tr);
        for (int i = 0; i < 4; ++i) tr->u[i] = ref_rng_peek(k0 + i);
        const Vertex* v1 = r->lat->GetVertices()[size_t(r->lat->GetNv() * tr->u[0])];
        const Vertex* v2 = v1->edges[size_t(v1->edges.size() * tr->u[1])]->GetOther(v1);
        tr->v1 = int32_t(v1->idx);
        tr->v2 = int32_t(v2->idx);
        bool up1 = before[0][v1->idx] != r->sp->GetNpt()[0];
        bool up2 = before[0][v2->idx] != r->sp->GetNpt()[0];
        tr->kind = (up1 != up2) ? 1 : 0;
        tr->accepted = r->step->stepped ? 1 : 0;
        BigDouble nw = r->step->inner.m_prev_weight;   // trystep's return value
        tr->w_new_c = nw.m_c;
        tr->w_new_e = nw.m_e;
        tr->ratio = double(nw / sw);
        tr->khop = -2;
    }
    return ORC_OK;
}

}  // namespace

extern "C" {

void* ref_create(int L, double phi, double neel, double neel_exp, double bcx, double bcy,
                 int channel, int qx, int qy, int* status)
{
    RefRun* r = new RefRun;
    r->L = L;
    r->channel = channel;
    r->fm = new FileManager(".", std::string("oracle"));
    r->fm->Verbose() = 0;
    r->lat = new SquareLattice(L, L);
    size_t LL = size_t(L) * L;
    std::vector<double> bc = {bcx, bcy};
    std::vector<size_t> Q = {size_t(qx), size_t(qy)};
    try {
        if (channel == ORC_CH_TRANS) {
            r->sp = new LatticeState(r->fm, r->lat, {LL / 2 + 1, LL / 2 - 1}, {1, 1});
            r->wav = new StagFluxTransExciton(r->fm, L, L, phi, neel, neel_exp, bc, Q);
        } else if (channel == ORC_CH_LONG) {
            r->sp = new LatticeState(r->fm, r->lat, {LL / 2, LL / 2}, {1, 1});
            r->wav = new StagFluxLongExciton(r->fm, L, L, phi, neel, neel_exp, bc, Q);
        } else {
            r->sp = new LatticeState(r->fm, r->lat, {LL / 2, LL / 2}, {1, 1});
            r->wav = new StagFluxGroundState(r->fm, L, L, phi, neel, neel_exp, bc);
        }
        r->amp = new SlaterDeterminant(r->sp, r->wav);
    } catch (std::exception&) {
        if (status) *status = ORC_ERR_INVALID;
        return nullptr;
    }
    if (status) *status = ORC_OK;
    return r;
}

void ref_destroy(void* h)
{
    RefRun* r = static_cast<RefRun*>(h);
    if (!r) return;
    teardown_chain(r);
    delete r->amp; delete r->wav; delete r->sp; delete r->lat; delete r->fm;
    delete r;
}

void ref_info(void* h, int* Ns, int* Nup, int* Ndn, int* Nexc)
{
    RefRun* r = static_cast<RefRun*>(h);
    *Ns = int(r->lat->GetNv());
    *Nup = int(r->sp->GetNpt()[0]);
    *Ndn = int(r->sp->GetNpt()[1]);
    *Nexc = int(r->wav->GetNExc());
}

void ref_phi(void* h, int fl, double* out)
{
    RefRun* r = static_cast<RefRun*>(h);
    size_t Ns = r->lat->GetNv();
    for (size_t f = 0; f < Ns; ++f)
        for (size_t x = 0; x < Ns; ++x) {
            std::complex<double> v = r->wav->MatEl(f, x, fl);
            out[2 * (f * Ns + x)] = v.real();
            out[2 * (f * Ns + x) + 1] = v.imag();
        }
}

void ref_neighbours(void* h, int32_t* nbr)
{
    RefRun* r = static_cast<RefRun*>(h);
    for (size_t v = 0; v < r->lat->GetNv(); ++v) {
        const Vertex* vx = r->lat->GetVertices()[v];
        for (size_t e = 0; e < 4; ++e) nbr[v * 4 + e] = int32_t(vx->edges[e]->GetOther(vx)->idx);
    }
}

void ref_orbitals(void* h, int fl, int32_t* orb)
{
    RefRun* r = static_cast<RefRun*>(h);
    for (size_t p = 0; p < r->wav->GetNpt()[fl]; ++p) orb[p] = int32_t(r->wav->Getpt()[fl][p]);
}

int ref_set_config(void* h, uint64_t seed, uint32_t walker, const int8_t* up)
{
    RefRun* r = static_cast<RefRun*>(h);
    r->seed = seed;
    r->walker = walker;
    size_t Ns = r->lat->GetNv();
    std::vector<std::vector<int>> fock(2, std::vector<int>(Ns, 0));
    for (size_t v = 0; v < Ns; ++v) { fock[0][v] = up[v] ? 1 : 0; fock[1][v] = up[v] ? 0 : 1; }
    try {
        r->sp->FockInit(fock);
        r->amp->Init();
        return finish_start(r);
    } catch (std::exception&) {
        return ORC_ERR_SINGULAR;
    }
}

int ref_random_start(void* h, uint64_t seed, uint32_t walker)
{
    RefRun* r = static_cast<RefRun*>(h);
    r->seed = seed;
    r->walker = walker;
    size_t L = r->L;
    std::vector<std::vector<size_t>> pop;
    if (r->channel == ORC_CH_TRANS) {
        pop.push_back(std::vector<size_t>(1, L * L / 2 + 1));
        pop.push_back(std::vector<size_t>(1, L * L / 2 - 1));
    } else {
        pop.push_back(std::vector<size_t>(1, L * L / 2));
        pop.push_back(std::vector<size_t>(1, L * L / 2));
    }
    ref_rng_set(seed, walker, 1, 0);
    int tc = 0, failcount = 10;
    try {
        while (r->amp->Amp() == 0.0 && tc < failcount) {     // vmc.cpp:230-234
            r->sp->RanInit(pop);
            r->amp->Init();
            tc++;
        }
        if (tc == failcount) return ORC_ERR_SINGULAR;
        return finish_start(r);
    } catch (std::exception&) {
        return ORC_ERR_SINGULAR;
    }
}

void ref_rng_seek(void* h, uint64_t k) { static_cast<RefRun*>(h)->next = k; }

int ref_step(void* h, int meas, orc_trace* tr) { return one_step(static_cast<RefRun*>(h), meas, tr); }

int ref_measure(void* h, int mask)
{
    RefRun* r = static_cast<RefRun*>(h);
    try {
        if (mask & ORC_MEAS_PROJHEIS) r->pj->measure();
        if (mask & ORC_MEAS_STAGMAGN) r->sm->measure();
        if (mask & ORC_MEAS_STATSPIN) r->ss->measure();
    } catch (std::exception&) {
        return ORC_ERR_SINGULAR;
    }
    return ORC_OK;
}

void ref_reset_quantities(void* h)
{
    RefRun* r = static_cast<RefRun*>(h);
    r->pj->init(); r->sm->init(); r->ss->init();
}

int ref_reinit(void* h)
{
    RefRun* r = static_cast<RefRun*>(h);
    r->amp->Init();
    r->reinversions++;
    r->since_reinv = 0;
    return r->amp->Amp() == 0.0 ? ORC_ERR_SINGULAR : ORC_OK;
}

// MetroMC::Walk itself when no per-step trace or re-inversion is requested;
// otherwise the same cadence (MetroMC.cpp:49-68) step by step.
int ref_walk(void* h, uint64_t len, uint64_t meas, int mask, int reinv_every, orc_trace* traces)
{
    RefRun* r = static_cast<RefRun*>(h);
    select_quantities(r, mask);
    if (!traces && reinv_every <= 0) {
        ref_rng_set(r->seed, r->walker, 0, r->next);
        try {
            r->mc->Walk(len, meas);
        } catch (std::exception&) {
            return ORC_ERR_SINGULAR;
        }
        r->next = ref_rng_next();
        return ORC_OK;
    }
    if (meas) for (Quantity* q : r->mc->GetQuantities()) q->init();
    for (uint64_t s = 0; s < len; ++s) {
        int rc = one_step(r, meas != 0, traces ? &traces[s] : nullptr);
        if (rc) return rc;
        if (reinv_every > 0 && r->since_reinv >= uint64_t(reinv_every)) {
            rc = ref_reinit(h);
            if (rc) return rc;
        }
        if (meas && (meas == 1 || s % meas == 0))
            for (Quantity* q : r->mc->GetQuantities()) q->measure();
    }
    return ORC_OK;
}

void ref_config(void* h, int8_t* up)
{
    RefRun* r = static_cast<RefRun*>(h);
    for (size_t v = 0; v < r->lat->GetNv(); ++v) up[v] = r->sp->Getfs()[0][v] != r->sp->GetNpt()[0];
}

void ref_particles(void* h, int fl, int32_t* part)
{
    RefRun* r = static_cast<RefRun*>(h);
    for (size_t p = 0; p < r->sp->GetNpt()[fl]; ++p) part[p] = int32_t(r->sp->Getpt()[fl][p]);
}

void ref_amp(void* h, double* mant, int32_t* e)
{
    BigComplex a = static_cast<RefRun*>(h)->amp->Amp();
    mant[0] = a.m_c.real(); mant[1] = a.m_c.imag(); *e = a.m_e;
}

void ref_weight(void* h, double* mant, int32_t* e)
{
    BigDouble w = static_cast<const Stepper*>(static_cast<RefRun*>(h)->step)->weight();
    *mant = w.m_c; *e = w.m_e;
}

void ref_inverse(void* h, int fl, double* out)
{
    RefRun* r = static_cast<RefRun*>(h);
    const std::vector<std::complex<double>>& m = r->amp->m_mati[fl];
    for (size_t i = 0; i < m.size(); ++i) { out[2 * i] = m[i].real(); out[2 * i + 1] = m[i].imag(); }
}

int ref_current_state(void* h) { return int(static_cast<RefRun*>(h)->wav->GetCurrentStateIndex()); }

void ref_counts(void* h, uint64_t* steps, uint64_t* rej, uint64_t* acc, uint64_t* reinv)
{
    RefRun* r = static_cast<RefRun*>(h);
    if (steps) *steps = r->mc->m_steps;
    if (rej) *rej = r->mc->m_rejection;
    if (acc) *acc = r->accepted_real;
    if (reinv) *reinv = r->reinversions;
}

int ref_projheis(void* h, double* vals)
{
    RefRun* r = static_cast<RefRun*>(h);
    for (size_t i = 0; i < r->pj->m_vals.size(); ++i) {
        vals[2 * i] = r->pj->m_vals[i].real();
        vals[2 * i + 1] = r->pj->m_vals[i].imag();
    }
    return r->pj->GetNmeas();
}

int ref_stagmagn(void* h, double* val)
{
    RefRun* r = static_cast<RefRun*>(h);
    val[0] = r->sm->m_vals.real(); val[1] = r->sm->m_vals.imag();
    return r->sm->GetNmeas();
}

int ref_statspin(void* h, double* vals)
{
    RefRun* r = static_cast<RefRun*>(h);
    for (size_t i = 0; i < r->ss->m_vals.size(); ++i) {
        vals[2 * i] = r->ss->m_vals[i].real();
        vals[2 * i + 1] = r->ss->m_vals[i].imag();
    }
    return r->ss->GetNmeas();
}

int ref_virt_update(void* h, int nset, const int32_t* hops, double* out)
{
    RefRun* r = static_cast<RefRun*>(h);
    std::vector<std::vector<hop_path_t>> rhop(nset, std::vector<hop_path_t>(2));
    for (int i = 0; i < nset; ++i)
        for (int fl = 0; fl < 2; ++fl)
            if (hops[4 * i + 2 * fl] >= 0)
                rhop[i][fl].push_back(hop_t(size_t(hops[4 * i + 2 * fl]), size_t(hops[4 * i + 2 * fl + 1])));
    std::vector<BigComplex> qs;
    try {
        r->amp->VirtUpdate(rhop, r->wav->GetHops(), qs);
    } catch (std::exception&) {
        return ORC_ERR_SINGULAR;
    }
    for (size_t i = 0; i < qs.size(); ++i) {
        out[3 * i] = qs[i].m_c.real();
        out[3 * i + 1] = qs[i].m_c.imag();
        out[3 * i + 2] = qs[i].m_e;
    }
    return ORC_OK;
}

}  // extern "C"
