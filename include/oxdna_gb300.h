/*
 * oxdna_gb300.h - C ABI of the GB300 (sm_103a) oxDNA / oxRNA force engine.
 *
 * Plain C: every entry point takes plain pointers, sizes and an opaque CUDA stream
 * (void*, a cudaStream_t; NULL = the legacy default stream). No C++ or torch types
 * cross this boundary. Every function returns an int status (OXG_OK = 0).
 *
 * Two levels are exported.
 *
 *  1. Evaluator level: the drop-in for the reference plugin's GPU force drivers.
 *     A HOOMD-side wrapper owns all particle buffers and hands device pointers in:
 *       oxg_pair_forces    replaces gpu_compute_pair_aniso_forces<EvaluatorPairOxDNA*>
 *                          (src/AnisoPotentialPairOxDNA*GPUKernel.cu:14-18), one call
 *                          for any subset of the six nonbonded evaluators;
 *       oxg_bonded_forces  replaces kernel::gpu_compute_oxdna_bonded_forces
 *                          (src/OxDNABondedGPU.cu:125-159) together with
 *                          OxDNABondedForceComputeGPU::computeForces/reduceSplit
 *                          (src/OxDNABondedForceComputeGPU.cc:51-101).
 *     Parameter setters replace the pybind dict -> param_type constructors
 *     (e.g. src/EvaluatorPairOxDNAHBondCross.h:69-101, src/OxDNABondedParams.h:97-127).
 *
 *  2. System level: a self-contained engine (state + cell neighbour list + fused
 *     force kernels + Langevin / NO_SQUISH integrator, CUDA-graph captured) that
 *     stands in for the HOOMD runtime the reference plugin runs inside.
 *
 * Data layout (device, structure of arrays, 16-byte aligned):
 *   pos_type[4*N]  x, y, z, type   The evaluator-level calls take HOOMD's Scalar4
 *                                   (double) arrays with the type in .w as the int
 *                                   bit pattern of the low word (HOOMD's
 *                                   __scalar_as_int, src/OxDNABondedGPU.cu:51-53);
 *                                   the system engine keeps float4 with the type as
 *                                   the int bit pattern of the float.
 *   quat[4*N]      w, x, y, z      (HOOMD Scalar4 quaternion order: s in .x)
 *   charge[N]      per-particle charge (Debye-Hueckel only)
 *   force[4*N]     fx, fy, fz, per-particle energy (0.5 * pair energy to each end)
 *   torque[4*N]    tx, ty, tz, 0   (lab frame)
 *   virial[6*N]    xx, xy, xz, yy, yz, zz, component-major with pitch N (optional)
 * Per-term energies are FP64 sums reduced on the device.
 *
 * Sign conventions follow the reference evaluators: dr = r_i - r_j (minimum image),
 * the evaluator force is the force on i, torques are lab-frame
 * (src/OxDNAAnisoPair.h:91-105, src/OxDNABaseBase.h:233-235).
 */
#ifndef OXDNA_GB300_H
#define OXDNA_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------------- */
#define OXG_OK 0
#define OXG_ERR_INVALID_ARG 1    /* bad pointer, size, type index or term id        */
#define OXG_ERR_CUDA 2           /* a CUDA runtime call failed                       */
#define OXG_ERR_NLIST_OVERFLOW 3 /* neighbour / pair / cell capacity exceeded        */
#define OXG_ERR_BAD_INDEX 4      /* a bond or neighbour index outside [0, N)         */
#define OXG_ERR_TIMEOUT 5        /* a bounded device-side wait gave up               */
#define OXG_ERR_NO_PARAMS 6      /* a requested term has no parameters set           */
#define OXG_ERR_CAPACITY 7       /* a fixed-size resource is too small               */
#define OXG_ERR_NONFINITE 8      /* the state holds NaN/Inf (integrator blew up)     */

/* ---- nonbonded term ids (one per reference evaluator, getName() in brackets) - */
#define OXG_EXCVOL 0      /* EvaluatorPairOxDNAExcVol      [oxdna_excvol]        */
#define OXG_HBOND 1       /* EvaluatorPairOxDNAHBond       [oxdna_hbond]         */
#define OXG_CROSS 2       /* EvaluatorPairOxDNACrossStacking [oxdna_crossstacking] */
#define OXG_HBONDCROSS 3  /* EvaluatorPairOxDNAHBondCross  [oxdna_hbondcross]    */
#define OXG_COAX 4        /* EvaluatorPairOxDNACoaxStacking [oxdna_coaxstacking] */
#define OXG_DEBYE 5       /* EvaluatorPairOxDNADebye       [oxdna_debye]         */
#define OXG_N_PAIR_TERMS 6
#define OXG_TERM_BIT(t) (1u << (t))

/* bonded split energies (OxDNABondedForceCompute getFene/getBondedExcVol/getStacking) */
#define OXG_E_FENE 0
#define OXG_E_BEXC 1
#define OXG_E_STACK 2

/* ---- parameter PODs ---------------------------------------------------------
 * One struct per reference param_type, fields in the reference's order and units.
 * f4 sets are (A, B, T0, TS, TC); f5 sets are (A, B, XC, XS); f1 is
 * (a, r0, rlow, rhigh, rclow, rchigh, blow, bhigh); f2 is
 * (k, r0, rc, rlow, rhigh, rclow, rchigh, blow, bhigh).                         */

/* src/EvaluatorPairOxDNAExcVol.h:30-39. Site pair k: 0 back-back, 1 base-base,
 * 2 base(i)-back(j), 3 back(i)-base(j). */
typedef struct oxg_excvol_params {
    double eps;
    double base_site[3];
    double back_site[3];
    double sigma[4];
    double rstar[4];
    double b[4];
    double rc[4];
} oxg_excvol_params;

/* src/EvaluatorPairOxDNAHBond.h:30-36. eps == 0 disables the pair (non-complementary). */
typedef struct oxg_hbond_params {
    double eps;
    double shift_factor;
    double base_site[3];
    double f1[8];
    double t1[5], t23[5], t4[5], t78[5];
} oxg_hbond_params;

/* src/EvaluatorPairOxDNACrossStacking.h:30-37. t4_enabled = 0 drops f4(theta4) (oxRNA). */
typedef struct oxg_cross_params {
    double base_site[3];
    double f2[9];
    double t1[5], t23[5], t4[5], t78[5];
    int32_t t4_enabled;
    int32_t pad_;
} oxg_cross_params;

/* src/EvaluatorPairOxDNAHBondCross.h:37-47 (fused HB + cross-stacking). */
typedef struct oxg_hbondcross_params {
    double base_site[3];
    double eps;
    double shift_factor;
    double f1[8];
    double hb_t1[5], hb_t23[5], hb_t4[5], hb_t78[5];
    double f2[9];
    double cs_t1[5], cs_t23[5], cs_t4[5], cs_t78[5];
} oxg_hbondcross_params;

/* src/EvaluatorPairOxDNACoaxStacking.h:32-47. t1_mode 0 = oxDNA1 reflection,
 * 1 = oxDNA2 harmonic SA*(t-SB)^2; rna_coax selects the oxRNA two-dihedral form. */
typedef struct oxg_coax_params {
    double stack_site[3];
    double stack_back_ref[3];
    double gamma;
    double f2[9];
    double t1[5], t4[5], t56[5];
    double phi3[4];
    double phi4[4];
    int32_t t1_mode;
    int32_t pad0_;
    double t1_sa, t1_sb;
    int32_t phi3_enabled;
    int32_t rna_coax;
} oxg_coax_params;

/* src/EvaluatorPairOxDNADebye.h:28-31 (needs per-particle charge). */
typedef struct oxg_debye_params {
    double back_site[3];
    double minus_kappa, prefactor, b_smooth, rc, rhigh;
} oxg_debye_params;

/* src/OxDNABondedParams.h:35-73 (FENE + bonded excluded volume + DNA/RNA stacking).
 * Bonded exc-vol site pair k: 0 base-base, 1 base(A)-back(B), 2 back(A)-base(B).
 * st_eps[typeA][typeB] with A the 3' end of the bond, B = A's 5' neighbour. */
typedef struct oxg_bonded_params {
    double eps_backbone, r0_backbone, delta_backbone, delta2;
    double back_site[3];
    double base_site[3];
    double excl_eps;
    double bx_sigma[3], bx_rstar[3], bx_b[3], bx_rc[3];
    int32_t stacking_enabled;
    int32_t rna_stacking;
    double stack_site[3];
    double stack_back_ref[3];
    double st_gamma;
    double st_f1[9]; /* a, r0, rlow, rhigh, rclow, rchigh, blow, bhigh, shift_factor */
    double st_eps[4][4];
    double t4[5];    /* f4 theta4 */
    double t5[5];    /* f4 theta5 (== theta6) */
    double p1[4];    /* f5 phi1 (== phi2) */
    double stack_3_site[3], stack_5_site[3];
    double bbvector_3[3], bbvector_5[3];
    double tB1[5], tB2[5];
} oxg_bonded_params;

/* ---- level 1: evaluator-level drop-in ----------------------------------------- */
typedef struct oxg_context oxg_context;

/* Create a parameter context for n_types particle types on the current device.
 * Replaces the per-evaluator param GPUArray set-up done by HOOMD's AnisoPotentialPair
 * and OxDNABondedForceComputeGPU (src/OxDNABondedForceComputeGPU.cc:18-38). */
int oxg_create(oxg_context** out, int n_types, int n_bond_types);
int oxg_destroy(oxg_context* ctx);

/* Set one unordered type pair (both (ti,tj) and (tj,ti) are written) and the COM
 * cutoff r_cut of that term. Mirrors params[(t1,t2)] = dict(...) with
 * default_r_cut (oxdna/forces.py:129-311, oxdna/model/dna2.py:100-204). */
int oxg_set_excvol_params(oxg_context* ctx, int ti, int tj, const oxg_excvol_params* p, double r_cut);
int oxg_set_hbond_params(oxg_context* ctx, int ti, int tj, const oxg_hbond_params* p, double r_cut);
int oxg_set_cross_params(oxg_context* ctx, int ti, int tj, const oxg_cross_params* p, double r_cut);
int oxg_set_hbondcross_params(oxg_context* ctx, int ti, int tj, const oxg_hbondcross_params* p, double r_cut);
int oxg_set_coax_params(oxg_context* ctx, int ti, int tj, const oxg_coax_params* p, double r_cut);
int oxg_set_debye_params(oxg_context* ctx, int ti, int tj, const oxg_debye_params* p, double r_cut);
/* OxDNABondedForceCompute::setParams (src/OxDNABondedForceCompute.cc:39-45). */
int oxg_set_bonded_params(oxg_context* ctx, int bond_type, const oxg_bonded_params* p);

/* Nonbonded forces over a HOOMD-layout FULL neighbour list (each pair listed from both
 * ends): neighbours of i are nlist[head_list[i] + k], k < n_neigh[i]. Evaluates the
 * terms in term_mask (OXG_TERM_BIT(...)) and ADDS into force/torque/virial (the caller
 * zeroes them, as HOOMD's net-force sum would). One warp per particle, lanes over
 * neighbours, warp-shuffle reductions, no atomics on force/torque.
 * term_energy (device, OXG_N_PAIR_TERMS doubles, may be NULL) receives the per-term
 * FP64 totals (ADDED). virial may be NULL. box = orthorhombic edge lengths.
 * HOOMD's FP64 positions, orientations and charges are first converted, a thread per
 * particle, into FP32 copies (positions as high + low parts, so differences keep FP64
 * accuracy) in a device buffer the context owns: allocated on the first call and grown
 * to the largest N seen (that growth synchronises `stream`).
 * The call is asynchronous on `stream`. A neighbour index outside [0, N) is skipped
 * and recorded; oxg_context_status() reports it (OXG_ERR_BAD_INDEX). */
int oxg_pair_forces(oxg_context* ctx, uint32_t term_mask, int N,
                    const double* pos_type, const double* quat, const double* charge,
                    const float box[3],
                    const uint32_t* n_neigh, const uint32_t* nlist, const uint64_t* head_list,
                    float* force, float* torque, float* virial, double* term_energy,
                    void* stream);

/* Bonded forces. bonds[3*b] = (A, B, bond_type) with B the 5' neighbour of A
 * (oxdna/io.py:219-220), device array. One thread per bond; ADDS into
 * force/torque/virial; split energies (device, 3 doubles: fene, bexc, stack, may be
 * NULL) are ADDED. virial may be NULL. Asynchronous; a bond with an index outside
 * [0, N) or an unknown bond type is skipped and recorded for oxg_context_status(). */
int oxg_bonded_forces(oxg_context* ctx, int N,
                      const double* pos_type, const double* quat, const float box[3],
                      int n_bonds, const int32_t* bonds,
                      float* force, float* torque, float* virial, double* split_energy,
                      void* stream);

/* Synchronise the context's last stream and return (and, if clear != 0, reset) the
 * first error recorded by the asynchronous device calls (OXG_OK when none). */
int oxg_context_status(oxg_context* ctx, int clear);

/* ---- level 2: system engine -------------------------------------------------- */
typedef struct oxg_system oxg_system;

/* Create a system of N particles (host arrays, copied to the device). bonds as in
 * oxg_bonded_forces (may be NULL when n_bonds == 0). The context's parameters are
 * read at every force evaluation, so they may be changed later. */
int oxg_system_create(oxg_system** out, oxg_context* ctx, int N, const float box[3],
                      int n_bonds, const int32_t* bonds_host);
int oxg_system_destroy(oxg_system* sys);
/* Work stream for every later call on this system (NULL = legacy default stream). */
int oxg_system_set_stream(oxg_system* sys, void* stream);
/* Host <-> device state transfer. Any pointer may be NULL to skip that array.
 * Positions are double-float: x = pos_type.xyz + pos_lo.xyz (pos_lo[4*N], .w unused;
 * NULL when setting = zero), which keeps ~1e-7 absolute precision in large boxes.
 * vel[4*N] = vx, vy, vz, mass; angmom[4*N] = quaternion conjugate momentum. */
int oxg_system_set_state(oxg_system* sys, const float* pos_type, const float* pos_lo,
                         const float* quat, const float* vel, const float* angmom,
                         const float* charge);
int oxg_system_get_state(oxg_system* sys, float* pos_type, float* pos_lo, float* quat,
                         float* vel, float* angmom);
/* Device pointers of the resident state (4*N floats each; charge N floats). A run
 * starts from the forces the previous run left for its final state when nothing has
 * changed since (as HOOMD's prepRun would recompute them); this call counts as a change.
 * After writing the state through these pointers later on, call oxg_system_set_state
 * with every array NULL so that the next run evaluates the forces again. */
int oxg_system_device_state(oxg_system* sys, float** pos_type, float** pos_lo, float** quat,
                            float** vel, float** angmom, float** charge);
/* Neighbour-list skin (HOOMD Cell nlist buffer, default 0.4). */
int oxg_system_set_nlist_buffer(oxg_system* sys, double buffer);
/* The system's timestep (0 after creation; every run advances it). The bath noise of
 * step t depends only on (seed, t, particle), so a state restored with its timestep
 * continues the noise stream: HOOMD's Simulation timestep restored from a snapshot. */
int oxg_system_set_timestep(oxg_system* sys, uint64_t step);
/* Evaluate forces at the current state: pair terms in term_mask plus (if bonded != 0)
 * the bonded force. Outputs are host arrays (any may be NULL): force/torque 4*N floats,
 * pair_energy OXG_N_PAIR_TERMS doubles, bonded_energy 3 doubles. */
int oxg_system_compute(oxg_system* sys, uint32_t term_mask, int bonded,
                       float* force, float* torque, double* pair_energy,
                       double* bonded_energy);
/* Langevin dynamics (velocity Verlet + NO_SQUISH rotation, gamma / gamma_r damping,
 * kT bath, counter-based RNG keyed by seed, step and particle).
 * Forces: pair terms in term_mask and the bonded force if bonded != 0. */
int oxg_system_set_integrator(oxg_system* sys, double dt, double kT, double gamma,
                              double gamma_r, uint64_t seed, uint32_t term_mask,
                              int bonded);
/* Advance nsteps steps (HOOMD run(): forces of the current state first, as prepRun; a
 * run that follows another run with nothing changed in between starts from the forces
 * that run left for the same state instead of evaluating them again). By default one
 * cooperative launch of the persistent run kernel per 2000 steps, one synchronisation
 * per launch; with OXG_RUN_MODE=graph in the environment at system creation, or while
 * a surrogate replaces the fused HB + cross-stacking term in MD steps, per-step kernels
 * replayed from captured CUDA graphs. On a neighbour-list overflow the lists grow and
 * the launch is replayed from its checkpoint. */
int oxg_system_run(oxg_system* sys, long nsteps);
/* One call for host-driven loops: load the state from the host arrays (pos_type,
 * pos_lo, quat, vel, angmom: float[4*N] each, as oxg_system_set_state), run nsteps >= 1
 * steps, and write the final state back into the same arrays. With page-locked, mapped
 * host arrays (cudaHostAlloc, torch pin_memory) on the persistent run kernel, the run
 * kernel itself reads the host arrays at its start (comparing them with the device
 * state: when they are equal and the last run left that state's forces, those are
 * reused) and its closing step writes the final state back: one launch per call, whose
 * end the host reads from a status word the launch writes into page-locked memory (or,
 * in a host session, no launch: see oxg_system_set_host_session). A particle type
 * outside the context's types is then
 * reported after the run (OXG_ERR_BAD_INDEX; the kernels skip the particle). Otherwise
 * set_state, run and get_state. No counterpart in the reference (HOOMD keeps the state
 * on the device between calls). */
int oxg_system_run_host(oxg_system* sys, long nsteps, float* pos_type, float* pos_lo, float* quat,
                        float* vel, float* angmom);
/* Host session for host-driven loops: with idle_us > 0, the run kernel of a
 * oxg_system_run_host call that takes one launch (nsteps <= 2000, page-locked arrays)
 * stays resident after the run, occupying every SM of the device, and serves the next
 * such call through a request block in page-locked host memory instead of a new launch
 * (~5 us instead of ~17 us of launch and completion on GB300); it leaves when no
 * request comes within idle_us microseconds (at most 100000), when any other call on
 * this system is made (each ends the session first), when the context's parameters
 * changed, or after a run that failed or overflowed its neighbour list (handled as
 * without a session). idle_us = 0 ends the session and turns it off (the default).
 * Other work on the device waits for the resident kernel to leave. No counterpart in
 * the reference. */
int oxg_system_set_host_session(oxg_system* sys, int idle_us);
/* Per-term energies at the current state (device reduction, FP64) into host arrays. */
int oxg_system_energies(oxg_system* sys, double* pair_energy, double* bonded_energy);
/* Counters: index 0 steps run, 1 neighbour-list builds, 2 pair-list entries (short),
 * 3 pair-list entries (long), 4 kernels launched per step, 5 host-state runs served by a
 * resident run kernel (oxg_system_set_host_session), 6 launches of the persistent run
 * kernel. */
int oxg_system_stats(oxg_system* sys, int64_t* out, int n);
/* Device time of the persistent run kernel measured with CUDA events around each of its
 * launches on the system's stream (those of oxg_system_run; oxg_system_run_host calls
 * are not timed): out[0] milliseconds, out[1] launches, out[2] step bodies, accumulated
 * since the last reset (reset != 0 clears after reading). */
int oxg_system_run_timing(oxg_system* sys, double* out, int n, int reset);

/* ---- learned surrogate of the fused HB + cross-stacking term -------------------
 * No counterpart in the reference: an extension. A 7 -> 64 -> 64 -> 64 -> 1 SiLU MLP per
 * pair class (complementary bases / the rest) maps the base-base geometry the plain
 * evaluator computes (BASE-BASE distance and the cosines c1, c2, c3, c4, c7, c8, in
 * that order) to the pair energy; forces and torques come from its analytic input
 * gradient. Weights are BF16 on the tensor cores with FP32 accumulation; FP32 master
 * parameters (OXG_MLP_PARAMS floats per class: W1[64][16] whose input columns 7..15
 * stay zero, b1[64], W2[64][64], b2[64], W3[64][64], b3[64], w4[64], b4, padding) are
 * trained by the library's own kernels. Inputs are normalised as (x - mu) * inv_sd and
 * the output is E = e_scale * y + e_shift.
 * Device-pointer arguments: feats[8*n] (7 raw features, class as 0/1), target[n],
 * idx[nb] (minibatch sample indices), y[n], dydx[7*n] (normalised units).            */
#define OXG_MLP_PARAMS 9480
typedef struct oxg_mlp oxg_mlp;
int oxg_mlp_create(oxg_mlp** out);
int oxg_mlp_destroy(oxg_mlp* m);
/* host arrays: 2 * OXG_MLP_PARAMS floats (class 0 then class 1) */
int oxg_mlp_set_params(oxg_mlp* m, const float* params);
int oxg_mlp_get_params(oxg_mlp* m, float* params);
int oxg_mlp_set_normalization(oxg_mlp* m, int cls, const float* mu, const float* inv_sd,
                              float e_scale, float e_shift);
/* gradient of L = sum_s (y_s - (target_s - e_shift) / e_scale)^2 / nb with respect to the
 * class's masters (host, OXG_MLP_PARAMS floats; NULL keeps it accumulated on the device)
 * and the sum of squared errors (host, may be NULL) */
int oxg_mlp_gradient(oxg_mlp* m, int cls, const float* feats, const float* target, const int* idx,
                     int nb, float* grad_host, double* sse_host, void* stream);
/* one Adam step (beta 0.9 / 0.999) of one class on a minibatch */
int oxg_mlp_train_step(oxg_mlp* m, int cls, const float* feats, const float* target,
                       const int* idx, int nb, float lr, double* sse_host, void* stream);
int oxg_mlp_predict(oxg_mlp* m, int cls, const float* feats, int n, float* y, float* dydx,
                    void* stream);

/* Surrogate use by a system. flags: OXG_SURROGATE_RUN replaces the fused HB + cross-
 * stacking pairs of MD steps (oxg_system_run), OXG_SURROGATE_COMPUTE those of
 * oxg_system_compute. Every audit_every MD steps (0 = never) a hashed 1 / audit_mod of
 * the pairs is also evaluated by the plain evaluator. The audited pairs are a sample of
 * the term's pairs, so (sum of the surrogate's pair energy errors) / (sum of the plain
 * pair energies) over them estimates the relative error of the term's energy; once at
 * least 100 pairs are audited, an estimate that exceeds audit_tol (a relative error,
 * e.g. 1e-4) by more than two standard errors switches the surrogate off (the plain
 * evaluator takes over) until the next set_surrogate. mlp = NULL or flags = 0 restores
 * the plain evaluator. */
#define OXG_SURROGATE_RUN 1
#define OXG_SURROGATE_COMPUTE 2
int oxg_system_set_surrogate(oxg_system* sys, const oxg_mlp* mlp, int flags, int audit_every,
                             int audit_mod, double audit_tol);
/* out[0..10]: disabled, audited pairs, audits that tripped the switch (0 or 1), rms
 * pair energy error, rms reference pair energy, rms force error, rms reference force,
 * max |pair energy error|, max |force error|, the sampled relative error of the term's
 * energy (sum of errors / sum of reference energies) and its standard error */
int oxg_system_surrogate_stats(oxg_system* sys, double* out, int n);
/* Training samples from the system's current state: every fused HB + CS pair that
 * passes the zero-factor tests gives feats[8*k..] (7 features, class) and the plain
 * evaluator's pair energy (device arrays of max_n samples); *n_out samples written. */
int oxg_system_hbx_samples(oxg_system* sys, int max_n, float* feats, float* energy, int* n_out);

/* ---- batched independent replicas ---------------------------------------------
 * No counterpart in the reference (which runs one HOOMD simulation per process):
 * R small systems stepped together in one persistent launch. Replica r has its own
 * context ctxs[r] (parameters, e.g. temperature-dependent stacking and Debye terms),
 * n_particles[r] particles, periodic box boxes[3r..3r+2], and n_bonds[r] bonds
 * (A, B, type) in replica-local indices, stored back to back in `bonds`. The state
 * arrays of oxg_batch_set_state / get_state hold the replicas back to back (replica
 * r starts at particle sum(n_particles[0..r-1])), in the oxg_system_set_state layout.
 * Replica r integrates with Langevin at kT[r] and Philox seed `seed + r`, so it
 * reproduces an oxg_system run of the same replica with that seed. Every pair of a
 * replica is tested (no neighbour list): meant for replicas of up to 512 particles.
 */
typedef struct oxg_batch oxg_batch;
int oxg_batch_create(oxg_batch** out, int n_replicas, oxg_context* const* ctxs,
                     const int32_t* n_particles, const float* boxes, const int32_t* n_bonds,
                     const int32_t* bonds);
int oxg_batch_destroy(oxg_batch* b);
int oxg_batch_set_stream(oxg_batch* b, void* stream);
/* host arrays, back to back over the replicas; NULL leaves a field unchanged */
int oxg_batch_set_state(oxg_batch* b, const float* pos_type, const float* pos_lo, const float* quat,
                        const float* vel, const float* angmom, const float* charge);
int oxg_batch_get_state(oxg_batch* b, float* pos_type, float* pos_lo, float* quat, float* vel,
                        float* angmom);
/* kT: n_replicas temperatures; mask/bonded select the terms as in oxg_system_set_integrator */
int oxg_batch_set_integrator(oxg_batch* b, double dt, const double* kT, double gamma,
                             double gamma_r, uint64_t seed, uint32_t term_mask, int bonded);
/* tile shape: at most tile_particles particles per CTA (1..512), threads 64/128/256 */
int oxg_batch_set_tiling(oxg_batch* b, int tile_particles, int threads);
/* time trial_steps for each admissible tile shape, keep the fastest (state unchanged) */
int oxg_batch_tune(oxg_batch* b, int trial_steps, int* tile_particles, int* threads,
                   double* best_ms);
int oxg_batch_run(oxg_batch* b, long nsteps);
/* host outputs: force[4N], torque[4N] (may be NULL), energies[9 * n_replicas] = per
 * replica the OXG_N_PAIR_TERMS pair-term totals then FENE, bonded excluded volume and
 * stacking */
int oxg_batch_compute(oxg_batch* b, uint32_t term_mask, int bonded, float* force,
                      float* torque, double* energies);

/* ---- allocation-free nonbonded evaluation -------------------------------------
 * No counterpart in the reference: an addition for callers that cannot allocate GPU
 * memory at all, e.g. code running inside a framework that has reserved the whole
 * device memory pool for its own allocator, or a host that forbids allocation (and
 * the implicit device synchronisation of cudaMalloc) once its simulation loop runs.
 *
 * Same evaluation as the system engine's nonbonded forces (cell list with bond
 * exclusions, split pair lists, the fused force kernel), but every scratch buffer it
 * needs lives in one fixed-size static device array inside this library (about
 * 18.1 MB, held by every GPU that loads the library until the process exits). The
 * call allocates nothing: no cudaMalloc, cudaFree or allocating library routine.
 *
 * Inputs (device): pos_type[4*N] (x, y, z, type as the float's int bits), quat[4*N],
 * charge[N] (NULL = unit charge), bonds[3*n_bonds] = (A, B, type) used for the
 * exclusions only. Outputs (device, overwritten): force[4*N] (F on each particle,
 * per-particle energy in .w when term_energy != NULL), torque[4*N], and term_energy
 * (OXG_N_PAIR_TERMS doubles, per-term totals; may be NULL). Parameters come from ctx
 * (its own device memory is not used).
 *
 * Limits: N <= OXG_NOALLOC_MAX_PARTICLES and n_bonds <= 2 * that, rejected with
 * OXG_ERR_CAPACITY before any GPU work; at most 64 particles per cell, 32 short-range
 * and 48 long-range neighbour pairs per allowed particle on average, at most 4 bonds
 * per particle: exceeding these is reported as OXG_ERR_CAPACITY after the run (the
 * call waits for its work on `stream` to finish before returning).
 *
 * The call copies its parameter block from host memory and reads its status back, so
 * it synchronises `stream` before returning and cannot be captured into a CUDA graph.
 * The first call on a device looks up the array's device address (once per device,
 * with that device current, and again after the device's context was replaced, e.g.
 * by cudaDeviceReset). Every call uses the same array and leaves its contents
 * behind; the call clears what must start empty. Calls whose GPU work overlaps
 * (several streams or threads) race on the shared array. */
#define OXG_NOALLOC_MAX_PARTICLES 8192
int oxg_pair_forces_noalloc(oxg_context* ctx, uint32_t term_mask, int N,
                            const float* pos_type, const float* quat, const float* charge,
                            const float box[3], int n_bonds, const int32_t* bonds,
                            float* force, float* torque, double* term_energy, void* stream);

/* Measured throughput of the current device's FP32 FMA pipe (out[0], GFLOP/s, an FMA
 * counted as two flops) and special-function unit (out[1], reciprocal square roots in
 * Gop/s): the denominators of the MD step's compute roofline. Runs two short
 * microbenchmark kernels (a few ms each) on `stream` and synchronises. n: entries of
 * `out` to fill (1 or 2). No counterpart in the reference: measurement support. */
int oxg_device_peaks(double* out, int n, void* stream);

/* Bounded-wait self-test of the run kernel's grid barrier: one cooperative launch of
 * n_blocks (2..64, at most the SM count) blocks meets at one barrier, except block
 * skip_block (none if negative), which never arrives. The others then give up after
 * the barrier's poll limit (about 1 s on a GB300) and the call returns OXG_ERR_TIMEOUT, the status
 * the run entry points return when a run kernel's barrier gives up; with no skipped
 * block it returns OXG_OK. results[b] (host, n_blocks entries): 1 passed the barrier,
 * 0 gave up, -1 skipped. The context stays usable either way. Failure-handling test
 * support; no counterpart in the reference. */
int oxg_selftest_barrier(int n_blocks, int skip_block, int* results, void* stream);

/* Text of the last error raised on the calling thread (CUDA error string etc.). */
const char* oxg_last_error(void);
/* Version / build string of the loaded library. */
const char* oxg_version(void);
/* Human-readable text for a status code. */
const char* oxg_status_string(int status);

#ifdef __cplusplus
}
#endif
#endif /* OXDNA_GB300_H */
