/*
 * gpvmc_gb300.h -- C ABI of the GB300 engine for the gpvmc Metropolis
 * sampling path (Gutzwiller-projected staggered-flux Slater determinants,
 * nearest-neighbour spin-exchange moves, ProjHeis / StagMagnZ /
 * StatSpinStruct measurements).
 *
 * Plain pointers and sizes only.  Every function returns a gv_status (0 =
 * GV_OK); nothing aborts.  A job owns its device memory and its CUDA stream;
 * the caller owns the job handle.  Calls on one job are not thread-safe;
 * distinct jobs may be driven from distinct host threads.
 *
 * The reference interfaces these entry points replace (reference files,
 * EPFL-LQM/gpvmc):
 *   gv_job_create          StagFlux{GroundState,TransExciton}::ctor + SquareLattice ctor +
 *                          LatticeState ctor + SlaterDeterminant ctor
 *                          (vmc.cpp:140-160; SlaterDeterminant.cpp:21-55)
 *   gv_job_init_walkers    LatticeState::FockInit / RanInit + SlaterDeterminant::Init +
 *                          excited-state arg-max + MetroMC ctor weight()
 *                          (vmc.cpp:161-263; LatticeState.cpp:37-113;
 *                          SlaterDeterminant.cpp:60-92; MetroMC.cpp:17-25)
 *   gv_job_walk            MetroMC::Walk(len, meas) with the attached quantities
 *                          (MetroMC.cpp:45-88 -> MetroMC::Step 90-103 ->
 *                          LatticeStepper::trystep/step LatticeStepper.cpp:36-147 ->
 *                          SlaterDeterminant::VirtUpdate/Update SlaterDeterminant.cpp:96-326)
 *   gv_job_reinvert        SlaterDeterminant::Init (SlaterDeterminant.cpp:60-92)
 *   gv_job_virt_update     SlaterDeterminant::VirtUpdate (SlaterDeterminant.cpp:96-268)
 *   gv_job_read_*          LatticeState::Getfs, SlaterDeterminant::Amp,
 *                          MetroMC::Rejection, Quantity m_vals / GetNmeas
 *                          (State.cpp:55-63; SlaterDeterminant.cpp:94;
 *                          MetroMC.cpp:105-111; Quantity.h:12-28)
 *   gv_job_checkpoint /    State::Save of the final Fock state and the --spinstate
 *   gv_job_restore         resume (State.cpp:117-166; vmc.cpp:178-220, 329)
 */
#ifndef GPVMC_GB300_H
#define GPVMC_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t gv_status;
#define GV_OK 0
#define GV_ERR_INVALID 1      /* bad argument / unsupported configuration */
#define GV_ERR_SINGULAR 2     /* no non-singular start, or singular update (linalg.cpp:23, 562-570) */
#define GV_ERR_NAN 3          /* NaN/Inf met (BigComplex.h:24-31, StagFluxWaveFunction.cpp:65-77) */
#define GV_ERR_ZERO_AMP 4     /* stepped to a zero overlap (LatticeStepper.cpp:121-124) */
#define GV_ERR_DRIFT 5        /* inverse drift above threshold after re-inversion */
#define GV_ERR_TIMEOUT 6      /* a bounded device wait gave up */
#define GV_ERR_OOM 7          /* device allocation failed */
#define GV_ERR_CUDA 8         /* other CUDA runtime error */
#define GV_ERR_NOT_READY 9    /* walkers not initialised */
#define GV_ERR_TOO_LARGE 10   /* size beyond a fixed-size entry point's limit */

#define GV_CH_GROUNDSTATE 0   /* StagFluxGroundState */
#define GV_CH_TRANS 1         /* StagFluxTransExciton */
#define GV_CH_LONG 2          /* StagFluxLongExciton */

#define GV_PREC_FP64 0        /* plain form: FP64 inverses, FP64 Sherman-Morrison */
#define GV_PREC_MIXED 1       /* FP32 inverses/updates, FP64 periodic re-inversion */

#define GV_FLAG_REINV_DEFERRED 1  /* re-invert walkers that reached reinv_every accepted
                                     exchanges at the end of each gv_job_walk call (one
                                     batched launch) rather than right after the move */
#define GV_FLAG_REINV_ON_DRIFT 2  /* with GV_FLAG_REINV_DEFERRED: at that point check the
                                     FP64 sampled drift ||A A^-1 - I||_max and re-invert
                                     only when it exceeds drift_threshold */
#define GV_FLAG_DELAYED_UPDATES 4 /* delayed Sherman-Morrison updates: the inverse is
                                     written back once per 4 accepted exchanges (the same
                                     Markov chain; the inverse differs only by rounding) */
#define GV_FLAG_STREAM_INVERSES 8 /* mixed ground state: keep the inverses in HBM during the
                                     walk (the streaming kernel) instead of on chip; the
                                     on-chip kernel runs by default when N <= 128 and the
                                     re-inversion is deferred */
#define GV_FLAG_CUDA_GRAPHS 32    /* capture each distinct walk call (len, meas, measured
                                     quantities) into a CUDA graph once and replay it: one
                                     launch per call instead of one per kernel (not while a
                                     job timer runs or a walk is traced) */
#define GV_FLAG_TC_PROJHEIS 64    /* mixed ground state, N <= 128: ProjHeis from the split-TF32
                                     tensor-core products G = Phi A^-1 of every antiparallel
                                     pair (the nearest-neighbour pairs are the bonds) instead
                                     of the per-particle FP32 dot products in the walk kernel;
                                     GV_ERR_INVALID at creation where it does not apply */
#define GV_FLAG_SCALAR_PAIRS 16   /* mixed precision: StatSpinStruct pair ratios (ground state),
                                     the transverse exciton's ProjHeis overlap rows
                                     Z = GupT^T Phi and the longitudinal exciton's bond overlap
                                     sums Z_b = R^T C_b from FP32 dot products on the CUDA cores
                                     instead of split-TF32 tensor-core products (the tensor-core
                                     forms run by default when N_0 = N_1 <= 128, resp.
                                     Nexc, N_1 <= 128, N_0 <= 160, resp. N_0 = N_1 <= 128) */

#define GV_MEAS_PROJHEIS 1    /* ProjHeis (ProjHeis.cpp:40-158), Bx = 0 */
#define GV_MEAS_STAGMAGN 2    /* StagMagnZ (StagMagnZ.cpp:12-43) */
#define GV_MEAS_STATSPIN 4    /* StatSpinStruct (StatSpinStruct.cpp:16-135) */
#define GV_MEAS_STAGMAGN_TRACK 8   /* StagMagnTrack (StagMagnTrack.cpp:21-50): every measurement's
                                      staggered magnetisation, in order (gv_job_read_tracks) */
#define GV_MEAS_OVERLAP_TRACK 16   /* OverlapTrack (OverlapTrack.cpp:26-29): every measurement's
                                      stepper weight, as log10 (gv_job_read_tracks) */

typedef struct gv_job gv_job;

/* One VMC job: one wavefunction channel on an L x L lattice and n_walkers
 * independent Markov chains (the reference runs one chain per MPI rank,
 * vmc.cpp:119-127). */
typedef struct {
    int32_t L;                /* lattice side (vmc.cpp:69) */
    int32_t channel;          /* GV_CH_* (vmc.cpp:93, 147-154) */
    int32_t q[2];             /* exciton momentum qx, qy (vmc.cpp:73-74) */
    double phi;               /* staggered flux in radians: the CLI value times pi (vmc.cpp:120) */
    double neel;              /* Neel field (vmc.cpp:81) */
    double neel_exp;          /* Neel field exponent (vmc.cpp:82) */
    double phase_shift[2];    /* boundary phases in units of pi (vmc.cpp:83-84) */
    double phi_range[2];      /* if phi_range[1] > phi_range[0]: per-walker phi ~ U[lo, hi) (radians) */
    double neel_range[2];     /* if neel_range[1] > neel_range[0]: per-walker neel ~ U[lo, hi) */
    int32_t n_walkers;        /* independent chains in this job */
    int32_t precision;        /* GV_PREC_* */
    uint64_t seed;            /* Philox key (vmc.cpp:79, 119) */
    uint32_t walker_base;     /* Philox walker id of walker 0 */
    int32_t reinv_every;      /* re-invert after this many accepted exchanges, 0 = never */
    int32_t meas_mask;        /* GV_MEAS_* quantities measured by gv_job_walk when meas > 0 */
    int32_t flags;            /* GV_FLAG_* */
    double drift_threshold;   /* GV_FLAG_REINV_ON_DRIFT threshold (e.g. 1e-5) */
} gv_job_config;

/* Per-step record of one walker (parity traces). */
typedef struct {
    int32_t v1, v2;           /* proposal vertices (LatticeStepper.cpp:45-47) */
    int32_t kind;             /* 0 = same flavour (no-op), 1 = spin exchange */
    int32_t accepted;         /* MetroMC::YesNo outcome */
    int32_t khop;             /* arg-max channel state after the proposal, -1 for no-op */
    int32_t pad;
    double ratio;             /* Metropolis ratio fed to YesNo */
    double u4;                /* the uniform YesNo compared against */
} gv_trace;

/* Create / destroy. */
gv_status gv_job_create(const gv_job_config* cfg, gv_job** out);
gv_status gv_job_destroy(gv_job* job);
gv_status gv_job_dims(const gv_job* job, int32_t* Ns, int32_t* Nup, int32_t* Ndn, int32_t* Nexc);
/* Device bytes this job holds (admission by HBM footprint). */
gv_status gv_job_footprint(const gv_job_config* cfg, uint64_t* bytes);

/* Select the quantities measured by later gv_job_walk calls (MetroMC::AddQuantity,
 * MetroMC.h:31). */
gv_status gv_job_set_meas_mask(gv_job* job, int32_t meas_mask);

/* Quantity::measure on every walker's current configuration, without a
 * step, added to the sums (Quantity.cpp:24-27); gv_job_reset_quantities is
 * Quantity::init (Quantity.cpp:19-22). */
gv_status gv_job_measure(gv_job* job);
gv_status gv_job_reset_quantities(gv_job* job);
/* Largest sampled FP64 drift seen at a drift check, per walker, and the
 * number of checks that needed no re-inversion. */
gv_status gv_job_read_drift_checks(gv_job* job, double* drift_seen, uint64_t* checks_without_reinversion);

/* Bounded device waits.  The tensor-core kernels (StatSpinStruct pair
 * ratios, exciton overlap rows) wait on an mbarrier for their MMAs, and the
 * on-chip ground-state walk for its bulk (TMA) copies of the inverses and of
 * the proposals' phase rows, with a poll budget; when it runs out the
 * walker's status becomes GV_ERR_TIMEOUT, the kernel still lets the MMAs or
 * copies it issued finish before it frees its tensor memory, and the next
 * calls on the job run normally (gv_job_init_walkers clears the status).  polls < 0 restores the default (4194304 polls);
 * polls = 0 makes every such wait give up at once, which tests exercise.
 * Applies to kernels enqueued after the call (cached CUDA graphs are
 * dropped).  Diagnostic; it has no counterpart in the reference, whose
 * CPU code never waits on a device. */
gv_status gv_job_set_wait_limit(gv_job* job, int32_t polls);

/* Start configurations.  up: n_walkers x Ns bytes, 1 where flavour 0 sits
 * (LatticeState::FockInit), or NULL for the reference's random start with up
 * to 10 retries (vmc.cpp:221-241), drawn from Philox stream 1.  A
 * mixed-precision job also redraws a random start whose inverse has an entry
 * above 1e6 (its FP32 ratios would overflow on the first steps). */
gv_status gv_job_init_walkers(gv_job* job, const int8_t* up);

/* MetroMC::Walk(len, meas) on every walker: len Metropolis steps, the
 * requested quantities measured after steps s with s % meas == 0 (meas = 0:
 * no measurement).  Quantities are reset at the start of a measuring walk
 * (MetroMC.cpp:49-51).  Enqueued on the job's stream; returns immediately. */
gv_status gv_job_walk(gv_job* job, uint64_t len, uint64_t meas);
/* As gv_job_walk, but the quantity sums keep accumulating from the previous
 * call instead of restarting (a long MetroMC::Walk cut into pieces: with len
 * a multiple of meas the measurement points are the same). */
gv_status gv_job_walk_continue(gv_job* job, uint64_t len, uint64_t meas);
/* Autotuner: times the walk-kernel variants that compute this job's chain --
 *   0 HBM-streaming kernel, default CTA width (128 threads for N <= 128, else 256)
 *   1 HBM-streaming kernel, 256 threads
 *   2, 3 as 0, 1 with delayed updates (depth 4)
 *   4 on-chip kernel (inverses in TMEM; mixed ground state, N <= 128, deferred re-inversion)
 * on a scratch job of the same configuration (min(n_walkers, 4 x SMs)
 * walkers, `steps` timed steps per walker after as many warm-up steps; 0:
 * one sweep), applies the fastest to the job (its GV_FLAG_DELAYED_UPDATES /
 * GV_FLAG_STREAM_INVERSES bits and CTA width) and remembers the choice for
 * jobs of the same shape (device, L, channel, precision, other flags,
 * walkers rounded up to a power of two) in this process.  *choice = the
 * variant (-1: nothing to choose, e.g. the exciton channel); us_per_step[5]
 * (optional) = walk-kernel device microseconds per step of all scratch
 * walkers (re-inversions, the same under every variant, excluded), -1 for
 * variants not applicable or not timed (a remembered choice times nothing).
 * Call it before gv_job_init_walkers or between walks; the chain is the same
 * under every variant up to FP32 rounding. */
gv_status gv_job_autotune(gv_job* job, uint64_t steps, int32_t* choice, double* us_per_step);
/* GV_FLAG_CUDA_GRAPHS: graphs cached for this job (-1: the runtime refused a
 * capture and the job enqueues its kernels directly) and graph replays so far. */
gv_status gv_job_graph_stats(gv_job* job, int32_t* cached, int64_t* replays);
/* The job's CUDA stream (cudaStream_t), for callers that order their own work
 * after the job's kernels. */
gv_status gv_job_stream(gv_job* job, void** stream);
/* As gv_job_walk, also recording walker `walker`'s per-step trace into the
 * host array trace[len] (synchronous). */
gv_status gv_job_walk_traced(gv_job* job, uint64_t len, uint64_t meas, int32_t walker, gv_trace* trace);
/* Single-walker stepping, the reference's step-level API for one chain
 * (callers that drive MetroMC::Step themselves, or a Stepper of their own).
 * The walker's Metropolis stream is the one gv_job_walk draws from, so
 * stepping and walking can be mixed.  Slow path: every call synchronises.
 *   gv_job_trystep   LatticeStepper::trystep (LatticeStepper.cpp:36-100): draws
 *                    u1, u2, u3 of the walker's next step, proposes the
 *                    exchange v[0] = floor(Ns u1) <-> v[1] = its neighbour
 *                    floor(deg u2) (u3 drawn and unused), evaluates
 *                    SlaterDeterminant::VirtUpdate over every channel state
 *                    and returns the proposal's weight sum_k |q_k|^2 as
 *                    weight_mant * 2^weight_exp2 (the current weight for a
 *                    same-flavour proposal) and the arg-max channel state
 *                    khop (-1 for a same-flavour proposal).  The proposal
 *                    stays pending for gv_job_step.
 *   gv_job_yesno     MetroMC::YesNo (MetroMC.cpp:27-43) with the step's u4:
 *                    accepted = ratio > 1 ? u4 < 1 : u4 < ratio; moves the
 *                    stream to the next step and counts a rejection.
 *   gv_job_step      LatticeStepper::step (LatticeStepper.cpp:102-147): applies
 *                    the pending proposal -- the lattice hop, the wavefunction
 *                    hop to its arg-max state, SlaterDeterminant::Update of
 *                    both inverses (linalg::InvUpdate) and the amplitude -- with
 *                    the same kernel code as an accepted step of gv_job_walk.
 *   gv_job_update    LatticeState::Hop + WaveFunction::Hop + SlaterDeterminant::
 *                    Update (SlaterDeterminant.cpp:270-326) for a given
 *                    exchange hop = (up_from, up_to, dn_from, dn_to) with
 *                    up_to = dn_from and dn_to = up_from (all -1: nothing)
 *                    and channel state `state` (-1: the arg-max).
 *   gv_job_stepper_weight  LatticeStepper::weight (LatticeStepper.cpp:149-169):
 *                    sum_k |q_k|^2 as mant * 2^exp2. */
gv_status gv_job_trystep(gv_job* job, int32_t walker, int32_t* v, double* weight_mant, int32_t* weight_exp2,
                         int32_t* khop);
gv_status gv_job_yesno(gv_job* job, int32_t walker, double ratio, int32_t* accepted);
gv_status gv_job_step(gv_job* job, int32_t walker);
gv_status gv_job_update(gv_job* job, int32_t walker, const int32_t* hop, int32_t state);
gv_status gv_job_stepper_weight(gv_job* job, int32_t walker, double* mant, int32_t* exp2);

/* Wait for the job's stream; returns the first walker error status if any. */
gv_status gv_job_synchronize(gv_job* job);

/* SlaterDeterminant::Init on every walker: FP64 LU re-inversion of both
 * Slater matrices from the current configuration (also resets the drift). */
gv_status gv_job_reinvert(gv_job* job);
/* max |(A * A^-1 - I)_ij| per walker and flavour, FP64, out[walker*2 + fl]. */
gv_status gv_job_drift(gv_job* job, double* out);

/* SlaterDeterminant::VirtUpdate for `nset` real-space hop sets of walker
 * `walker`: hops[4*i..4*i+3] = (up_from, up_to, dn_from, dn_to) site
 * indices, -1 for no hop in that flavour.  For each set i and channel state k,
 * out[2*(k*nset+i)..+1] = det ratio product over flavours including the
 * channel-state hop sign, relative to the current amplitude (qs / Amp()). */
gv_status gv_job_virt_update(gv_job* job, int32_t walker, int32_t nset, const int32_t* hops, double* out);

/* Readers (synchronise the job's stream first). */
gv_status gv_job_read_config(gv_job* job, int8_t* up /* n_walkers x Ns */);
gv_status gv_job_read_particles(gv_job* job, int32_t walker, int32_t fl, int32_t* part /* N[fl] */);
/* Amplitude Amp() of each walker as a base-10 mantissa/exponent pair:
 * mant[2*w], mant[2*w+1] (re, im) with |mant| in [1,10), exp10[w]. */
gv_status gv_job_read_amplitude(gv_job* job, double* mant, int32_t* exp10);
/* Inverse Slater matrix of walker/flavour in the reference's column-major
 * layout (m_mati[p + f*N]) as interleaved complex doubles. */
gv_status gv_job_read_inverse(gv_job* job, int32_t walker, int32_t fl, double* out);
/* counts[w*5 + i]: steps, accepted exchanges, accepted no-ops, rejections,
 * re-inversions. */
gv_status gv_job_read_counts(gv_job* job, uint64_t* counts);
/* The wavefunction's Fock state of one walker and flavour (State::m_part):
 * orb[f] = orbital held by Slater row f (N[fl] entries; ground state: 2f). */
gv_status gv_job_read_orbitals(gv_job* job, int32_t walker, int32_t fl, int32_t* orb);
/* Status of every walker (GV_OK, or the error that stopped it; a stopped
 * walker takes no further steps until gv_job_init_walkers). */
gv_status gv_job_read_status(gv_job* job, int32_t* status /* n_walkers */);
/* WaveFunction::m_c_exc: current channel state of every walker (0 for the
 * ground state). */
gv_status gv_job_read_state_index(gv_job* job, int32_t* state /* n_walkers */);
/* LatticeStepper's weight (LatticeStepper.cpp:149-169) over |Amp()|^2 per
 * walker: sum over channel states k of |q_k / Amp()|^2 (1 for the ground state). */
gv_status gv_job_read_weight(gv_job* job, double* sigma /* n_walkers */);
/* Quantity sums since the last measuring walk began, per walker:
 * ProjHeis m_vals (2*Nexc*Nexc complex per walker; for the ground state
 * [E*L^2-normalised sum, count]), StagMagnZ (1 complex per walker), and the
 * job-wide StatSpinStruct sums (5*Ns*Ns complex: szz, s+-, s-+, s++, s--),
 * with the number of measurements each walker made.  A mixed exciton job sums
 * its H / O outer products in FP32 over blocks of 32 measurements before one
 * FP64 add per entry; the read folds a block still open into what it returns
 * and leaves the job's sums as they are. */
gv_status gv_job_read_projheis(gv_job* job, double* vals, int32_t* nmeas);
gv_status gv_job_read_stagmagn(gv_job* job, double* vals, int32_t* nmeas);
gv_status gv_job_read_statspin(gv_job* job, double* vals, int32_t* nmeas);

/* Track quantities (GV_MEAS_STAGMAGN_TRACK, GV_MEAS_OVERLAP_TRACK): room for
 * `capacity` measurements per walker (allocated here; 0 frees it); the tracks
 * restart with every measuring gv_job_walk (Quantity::init) and stop growing
 * when full.  gv_job_read_tracks copies, per walker, the staggered
 * magnetisation values stagmagn[w * capacity + i] (real; the reference's
 * complex value has zero imaginary part), log10 of the stepper weight
 * log10_weight[w * capacity + i] (|Amp|^2; exciton: sum_k |q_k|^2) -- the
 * reference's OverlapTrack::save divides the weights by their mean -- and the
 * number of entries n[w]; any pointer may be NULL.  Tracks are not part of a
 * checkpoint. */
gv_status gv_job_set_track_capacity(gv_job* job, int32_t capacity);
gv_status gv_job_read_tracks(gv_job* job, double* stagmagn, double* log10_weight, int32_t* n);

/* Checkpoint / resume.  The reference saves the final lattice Fock state
 * (State::Save, State.cpp:117-166) and resumes a chain from it with
 * --spinstate (vmc.cpp:178-220, LatticeState::FockInit), re-inverting and
 * drawing fresh random numbers.  A checkpoint here is a self-describing byte
 * blob holding, per walker, the particle order on the lattice, the
 * wavefunction's Fock state (exciton channel: slots, sign, channel state,
 * weight), the amplitude, the Philox counter, the step / acceptance /
 * re-inversion counters, the drift record, the status and the quantity sums,
 * behind a header with the job configuration and an FNV-1a checksum.
 *   GV_CKPT_INVERSES  also store the inverses (and exciton overlap rows) in
 *                     the job's precision: the restored job then continues
 *                     bit for bit as the checkpointed one would have.
 *                     Without it the restore re-inverts in FP64
 *                     (SlaterDeterminant::Init), which is what the
 *                     checkpointed job would give after gv_job_reinvert.
 * gv_job_checkpoint_size: bytes the blob needs.  gv_job_checkpoint waits for
 * the job's stream and writes the blob (GV_ERR_INVALID if capacity is short).
 * gv_job_restore loads a blob into a job created with the same lattice,
 * channel, walkers, seed, walker_base and wavefunction parameters (and, with
 * stored inverses, the same precision); any mismatch or a damaged blob is
 * GV_ERR_INVALID and leaves the job as it was.  The quantity sums continue
 * with gv_job_walk_continue. */
#define GV_CKPT_INVERSES 1
gv_status gv_job_checkpoint_size(gv_job* job, int32_t flags, uint64_t* bytes);
gv_status gv_job_checkpoint(gv_job* job, int32_t flags, void* buf, uint64_t capacity, uint64_t* written);
gv_status gv_job_restore(gv_job* job, const void* buf, uint64_t size);

/* CUDA-event timer on the job's stream: start records an event, stop
 * records another, waits for it and returns the elapsed milliseconds; the
 * launch count covers every kernel this job enqueued in between. */
gv_status gv_job_timer_start(gv_job* job);
gv_status gv_job_timer_stop(gv_job* job, double* ms, int64_t* launches);
/* Device time (CUDA events around each launch) spent between the last
 * timer start/stop in kernels of one kind: 0 Metropolis walk, 1 FP64
 * (re-)inversion, 2 measurement kernels; with their launch count. */
gv_status gv_job_kernel_ms(gv_job* job, int32_t kind, double* ms, int64_t* launches);
/* The individual launch durations behind gv_job_kernel_ms (up to capacity). */
gv_status gv_job_kernel_times(gv_job* job, int32_t kind, double* out, int64_t capacity, int64_t* n);

/* Device-time of the last gv_job_walk in milliseconds (CUDA events on the
 * job's stream) and the number of kernels it launched. */
gv_status gv_job_last_walk_ms(gv_job* job, double* ms, int64_t* launches);

/* Host-side tables (no device needed).
 * gv_phi_table: WaveFunction::MatEl cache m_cache[fl][o*Ns + s] of the
 *   staggered-flux orbitals (StagFluxWaveFunction.cpp:51-79; WaveFunction.cpp:27-37),
 *   interleaved complex doubles, Ns*Ns entries.
 * gv_lattice_neighbours: nbr[v*4 + e], e-th neighbour of v in LatticeStepper's
 *   draw order (SquareLattice.cpp:9-28; LatticeStepper.cpp:45-47).
 * gv_channel_orbitals: occupied orbitals of flavour fl in the channel's first
 *   state, by particle (row) index (StagFluxGroundState.cpp:3-15).
 * gv_philox4x32_10 / gv_uniform_at: the Philox4x32-10 stream every walker
 *   draws (counter {call_lo, call_hi, walker, stream}, key {seed_lo, seed_hi},
 *   uniform k from call k/2) -- stream 0 Metropolis, 1 start configuration,
 *   2 per-walker (phi, neel). */
gv_status gv_phi_table(int32_t L, double phi, double neel, double neel_exp, const double* phase_shift,
                       int32_t fl, double* out);
gv_status gv_lattice_neighbours(int32_t L, int32_t* nbr);
gv_status gv_channel_orbitals(int32_t L, const double* phase_shift, int32_t channel, const int32_t* q,
                              int32_t fl, int32_t* orb, int32_t* N, int32_t* Nexc);
/* gv_channel_states: the channel's state table, exciton channels only.
 * Transverse (StagFluxTransExciton.cpp:7-44): state k adds orbital exc_up[k]
 * to flavour 0 and removes orbital exc_dn[k] from flavour 1.  Longitudinal
 * (StagFluxLongExciton.cpp:6-66): state k < Ns replaces the lower-band
 * orbital exc_dn[k] by the upper-band orbital exc_up[k] in flavour k % 2 (the
 * other flavour fills the lower band); state Ns, present at q = 0 and
 * q = (L/2, L/2), is the ground state (-1, -1).  Nexc entries each. */
gv_status gv_channel_states(int32_t L, const double* phase_shift, int32_t channel, const int32_t* q,
                            int32_t* exc_up, int32_t* exc_dn);
/* gv_fock_quantum_numbers: out[3*f + 0..2] = (kx, ky, band) of every fock
 * orbital f < L*L, the integer labels StagFluxWaveFunction::quantum_numbers
 * reports (StagFluxWaveFunction.cpp:81-87) and WaveFunction::Save writes as
 * the states file's attributes (WaveFunction.cpp:85-137). */
gv_status gv_fock_quantum_numbers(int32_t L, const double* phase_shift, int32_t* out);
void gv_philox4x32_10(const uint32_t* ctr, const uint32_t* key, uint32_t* out);
double gv_uniform_at(uint64_t seed, uint32_t walker, uint32_t stream, uint64_t k);

/* Allocation-free inversion of one Slater matrix, for callers that cannot let
 * a library allocate device memory (applications that pre-allocate all of
 * their HBM at start-up and forbid later allocations, or latency-critical
 * loops where cudaMalloc's implicit synchronisation is not acceptable).  It
 * has no counterpart in the reference; it performs what linalg::DetInv does
 * for one matrix, in FP64 on the GPU.
 *   d_A    device, N x N complex (interleaved re, im) in the reference's
 *          column-major m_mat layout, A[r*N + f] = A(f, r); not modified
 *   d_Ai   device output, the inverse in the m_mati layout (N x N complex)
 *   d_info device output, 4 doubles (8-byte aligned): det mantissa (re, im),
 *          det base-2 exponent, status (GV_OK or GV_ERR_SINGULAR; singular:
 *          zero mantissa as linalg::DetInv, and d_Ai is not an inverse)
 * d_A and d_Ai must be 16-byte aligned; misaligned pointers are GV_ERR_INVALID
 * before anything is enqueued.
 *   stream cudaStream_t to enqueue on (NULL: the default stream)
 * The only working memory is a static device array sized for
 * N <= GV_NOALLOC_MAX_N (256 KiB, held by every GPU that loads the library
 * until exit); larger N returns GV_ERR_TOO_LARGE.  The call allocates and
 * frees nothing.  Its first call on a device looks up that array's device
 * address (make that first call before any stream capture).  All calls share
 * the array: calls that overlap on the GPU race and must be serialised.  The
 * looked-up address lives as long as the device's primary context: do not
 * call this entry point on a device after cudaDeviceReset. */
#define GV_NOALLOC_MAX_N 128
gv_status gv_slater_invert_noalloc(const double* d_A, double* d_Ai, int32_t N, double* d_info, void* stream);

/* Bytes this library has copied host -> device and device -> host since the
 * process loaded it (all jobs and threads), counted at every copy it issues:
 * end-to-end accounting of what a workload moves over the host link.  No
 * counterpart in the reference (a CPU program). */
gv_status gv_transfer_bytes(uint64_t* h2d, uint64_t* d2h);

/* Library version string. */
const char* gv_version(void);
/* Message for a status code. */
const char* gv_status_string(gv_status s);
/* The CUDA runtime's message for the last CUDA error this thread's calls into
 * the library met (behind a GV_ERR_CUDA / GV_ERR_OOM status), "" if none. */
const char* gv_last_cuda_error(void);

/* ---- Serving: a request loop with continuous batching -------------------
 * Requests (a job configuration plus thermalisation and measured sweeps) are
 * queued as they arrive; a host thread admits them in arrival order while the
 * device bytes of the admitted jobs (gv_job_footprint) stay within the budget
 * and a slot is free, keeps every admitted job's walkers resident on the
 * device, advances all admitted jobs concurrently (each on its own stream,
 * two walk calls of chunk_sweeps sweeps in flight per job, so their kernels
 * overlap on the GPU), and retires each job when its sweeps are done.  A job
 * depends only on its own request: its results are the same alone and in the
 * mix. */
typedef struct gv_server gv_server;

typedef struct {
    uint64_t hbm_budget;      /* device bytes the admitted jobs may hold; 0: 80% of the free memory */
    int32_t max_jobs;         /* jobs on the device at once */
    int32_t chunk_sweeps;     /* sweeps per walk call of a job (re-inversion checks run at call ends) */
} gv_server_config;

typedef struct {
    gv_job_config job;        /* wavefunction, walkers, precision, seed, re-inversion policy, meas_mask */
    uint64_t therm_sweeps;    /* sweeps (L*L steps) before measuring */
    uint64_t sweeps;          /* measured sweeps */
    uint64_t meas;            /* steps between measurements; divides L*L */
    int32_t validate;         /* 1: at the end compare one ProjHeis measurement with fresh FP64 inverses */
    int32_t pad;
} gv_request;

#define GV_REQ_PENDING 0
#define GV_REQ_RUNNING 1
#define GV_REQ_DONE 2

typedef struct {
    int32_t state;            /* GV_REQ_* */
    gv_status status;         /* the job's status once done */
    uint64_t steps;           /* Metropolis steps over all walkers, thermalisation included */
    uint64_t accepted;        /* accepted exchanges */
    uint64_t footprint;       /* device bytes the job was admitted with */
    double e_site;            /* ground state: mean over walkers of the ProjHeis E/site average;
                                 exciton: mean over walkers of Re tr H / (Ns Re tr O) */
    double stagmagn;          /* mean over walkers of the StagMagnZ average */
    double validation_error;  /* validate = 1: ground state max |dE/site| over walkers; exciton
                                 max |H,O - H,O(FP64)| / max |H,O(FP64)|; -1 otherwise */
    double t_submit, t_admit, t_done;   /* seconds since the server started */
    double t_started;         /* job created and walkers started (FP64 start inversions done) */
    double t_walked;          /* last walk call of the job complete on the device (0: never walked) */
} gv_result;

gv_status gv_server_create(const gv_server_config* cfg, gv_server** out);
/* Queue a request; returns its ticket.  GV_ERR_INVALID for a configuration
 * the engine rejects (checked at submission). */
gv_status gv_server_submit(gv_server* srv, const gv_request* req, uint64_t* ticket);
/* State and, once done, results of a request (non-blocking). */
gv_status gv_server_poll(gv_server* srv, uint64_t ticket, gv_result* out);
/* Wait until the request is done or timeout_s elapsed (GV_ERR_TIMEOUT). */
gv_status gv_server_wait(gv_server* srv, uint64_t ticket, double timeout_s, gv_result* out);
/* Wait until every submitted request is done (GV_ERR_TIMEOUT after timeout_s). */
gv_status gv_server_drain(gv_server* srv, double timeout_s);
/* Finish the admitted and queued requests, then stop the loop and free it. */
gv_status gv_server_destroy(gv_server* srv);

#ifdef __cplusplus
}
#endif
#endif
