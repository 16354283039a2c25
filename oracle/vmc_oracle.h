/*
 * vmc_oracle.h -- CPU restatement of the gpvmc Metropolis sampling path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the parity oracle: it restates, in
 * plain C, what the reference (EPFL-LQM/gpvmc) computes on its sampling hot
 * path.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
 * may load it, and only as the checker (or as the timed CPU baseline).  The
 * product (gpvmc_gb300/) never links, loads or calls anything in oracle/.
 *
 * Parity pin: the restatement is checked against the reference itself,
 * compiled unmodified from its sources by oracle/ref/Makefile with project
 * shims (stub HDF5 header, restated BLAS/LAPACK, Philox RanGen), through the
 * golden fixtures in tests/golden/ and, where the reference build exists, by
 * live comparison (tests/test_oracle_vs_ref.py).
 *
 * Every function cites the reference file:line it follows.
 */
#ifndef VMC_ORACLE_H
#define VMC_ORACLE_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_CH_GROUNDSTATE = 0, ORC_CH_TRANS = 1, ORC_CH_LONG = 2 };

enum {
    ORC_OK = 0,
    ORC_ERR_INVALID = 1,
    ORC_ERR_SINGULAR = 2,   /* no non-singular start / InvUpdate singular */
    ORC_ERR_NAN = 3,        /* BigComplex::bound NaN/Inf, matrix_element NaN */
    ORC_ERR_ZERO_AMP = 4,   /* LatticeStepper::step: stepped to zero overlap */
    ORC_ERR_WEIGHT = 5      /* LatticeStepper::step: weight self-check > 1e-6 */
};

enum { ORC_MEAS_PROJHEIS = 1, ORC_MEAS_STAGMAGN = 2, ORC_MEAS_STATSPIN = 4 };

typedef struct orc_job orc_job;
typedef struct orc_walker orc_walker;

/* Per-step trace record (one MetroMC::Step). */
typedef struct {
    int32_t v1, v2;          /* proposal vertices */
    int32_t kind;            /* 0 = same-flavour no-op, 1 = spin exchange */
    int32_t accepted;        /* 1 if MetroMC::YesNo accepted */
    int32_t khop;            /* arg-max wavefunction state (LatticeStepper::m_khop) */
    int32_t pad;
    double u[4];             /* the four uniforms drawn */
    double ratio;            /* double(new_weight / state_weight) as fed to YesNo */
    double w_new_c;          /* new weight (BigDouble mantissa, exponent) */
    int32_t w_new_e;
    int32_t pad2;
} orc_trace;

/* Philox4x32-10 (Salmon et al., SC'11) and the project's uniform mapping. */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
double orc_u01(uint32_t a, uint32_t b);
/* The k-th uniform (0-based) of stream (seed, walker, stream). */
double orc_uniform_at(uint64_t seed, uint32_t walker, uint32_t stream, uint64_t k);

/* Job = lattice + staggered-flux wavefunction of a channel.
 * phi is in radians (the value StagFluxWaveFunction receives, i.e. the CLI
 * value times pi, vmc.cpp:120).  bc = phase_shift_x/y (vmc.cpp:83-84). */
orc_job* orc_job_create(int L, double phi, double neel, double neel_exp,
                        double bcx, double bcy, int channel, int qx, int qy, int* status);
void orc_job_destroy(orc_job* job);
void orc_job_info(const orc_job* job, int* Ns, int* Nup, int* Ndn, int* Nexc);
/* m_cache[fl][f*Ns + r] as interleaved (re, im) doubles, Ns*Ns entries. */
void orc_job_phi(const orc_job* job, int fl, double* out);
/* Neighbour table nbr[v*4 + e] in LatticeStepper's draw order. */
void orc_job_neighbours(const orc_job* job, int32_t* nbr);
/* Orbitals occupied by the wavefunction's current (first) state, per flavour. */
void orc_job_orbitals(const orc_job* job, int fl, int32_t* orb);

orc_walker* orc_walker_create(orc_job* job, uint64_t seed, uint32_t walker_id);
void orc_walker_destroy(orc_walker* w);
/* Start from a spin configuration up[v] in {0,1} (LatticeState::FockInit +
 * SlaterDeterminant::Init + excited-state arg-max, vmc.cpp:178-254). */
int orc_walker_set_config(orc_walker* w, const int8_t* up);
/* Random S_z start with retries, uniforms from stream 1 (vmc.cpp:221-254). */
int orc_walker_random_start(orc_walker* w);
/* Reposition the Metropolis uniform stream (stream 0) at uniform index k. */
void orc_walker_rng_seek(orc_walker* w, uint64_t k);
/* One MetroMC::Step (MetroMC.cpp:90-103); trace may be NULL. */
int orc_walker_step(orc_walker* w, int meas, orc_trace* trace);
/* MetroMC::Walk (MetroMC.cpp:45-88) with the requested quantities; with
 * reinv_every > 0, SlaterDeterminant::Init is re-run after every reinv_every
 * accepted spin exchanges.  traces (len entries) may be NULL. */
int orc_walker_walk(orc_walker* w, uint64_t len, uint64_t meas, int meas_mask,
                    int reinv_every, orc_trace* traces);
int orc_walker_measure(orc_walker* w, int meas_mask);
void orc_walker_reset_quantities(orc_walker* w);
int orc_walker_reinit(orc_walker* w);

/* State readers. */
void orc_walker_config(const orc_walker* w, int8_t* up);
void orc_walker_particles(const orc_walker* w, int fl, int32_t* part);
void orc_walker_amp(const orc_walker* w, double* mant /*2*/, int32_t* exp10);
void orc_walker_weight(const orc_walker* w, double* mant, int32_t* exp10);
void orc_walker_inverse(const orc_walker* w, int fl, double* out /* N*N complex, column-major */);
int orc_walker_current_state(const orc_walker* w);
void orc_walker_counts(const orc_walker* w, uint64_t* steps, uint64_t* rejections,
                       uint64_t* accepted_real, uint64_t* reinversions);
/* Accumulated quantity sums (MatrixQuantity/ScalarQuantity m_vals) and m_meas. */
int orc_walker_projheis(const orc_walker* w, double* vals /* 2*Nexc*Nexc complex */);
int orc_walker_stagmagn(const orc_walker* w, double* val /* 1 complex */);
int orc_walker_statspin(const orc_walker* w, double* vals /* 5*Ns*Ns complex */);

/* SlaterDeterminant::VirtUpdate for nset real-space swap sets
 * hops[4*i .. 4*i+3] = (up_from, up_to, dn_from, dn_to), -1 = no hop in that
 * flavour, against all wavefunction states (khop = GetHops()).
 * out[(k*nset + i)] as (mant_re, mant_im, exp10) triples. */
int orc_walker_virt_update(const orc_walker* w, int nset, const int32_t* hops, double* out);

#ifdef __cplusplus
}
#endif
#endif
