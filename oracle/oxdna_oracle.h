/*
 * oxdna_oracle.h - FP64 CPU oracle for the oxDNA force hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This is the oracle: a plain-C, all-double restatement
 * of the reference plugin's per-pair evaluators, its bonded kernel and the HOOMD
 * driver semantics around them (minimum image, per-type-pair cutoffs, 0.5*E split,
 * Newton's third law, bond exclusions, Langevin + NO_SQUISH). Only the test suite,
 * the smoke check and the bench's CPU-baseline leg may load it; the GPU product never
 * links or calls it.
 *
 * Parity pin: every evaluator here is checked against the reference's own headers
 * compiled unchanged (oracle/ref_wrap.cpp, built into oracle/_ref/ by
 * oracle/build_ref.sh) through golden fixtures committed under tests/golden/.
 */
#ifndef OXDNA_ORACLE_H
#define OXDNA_ORACLE_H

#include <stdint.h>
#include "../include/oxdna_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- single-pair evaluators (HOOMD evaluate(): force on i, torques lab frame) --- */
/* Each returns 1 when rsq < rcutsq (HOOMD's "evaluated" flag), else 0 and zeros.  */
int oxo_excvol(const oxg_excvol_params* p, const double dr[3], const double qi[4],
               const double qj[4], double rcutsq, double f[3], double* e, double ti[3],
               double tj[3]);
int oxo_hbond(const oxg_hbond_params* p, const double dr[3], const double qi[4],
              const double qj[4], double rcutsq, double f[3], double* e, double ti[3],
              double tj[3]);
int oxo_cross(const oxg_cross_params* p, const double dr[3], const double qi[4],
              const double qj[4], double rcutsq, double f[3], double* e, double ti[3],
              double tj[3]);
int oxo_hbondcross(const oxg_hbondcross_params* p, const double dr[3], const double qi[4],
                   const double qj[4], double rcutsq, double f[3], double* e, double ti[3],
                   double tj[3]);
int oxo_coax(const oxg_coax_params* p, const double dr[3], const double qi[4],
             const double qj[4], double rcutsq, double f[3], double* e, double ti[3],
             double tj[3]);
int oxo_debye(const oxg_debye_params* p, const double dr[3], const double qi[4],
              const double qj[4], double rcutsq, double charge_i, double charge_j,
              double f[3], double* e, double ti[3], double tj[3]);

/* One bond (A, B = A's 5' neighbour); Rc = r_B - r_A (minimum image).
 * out: FB[3] force on B, tauA[3], tauB[3], e[3] (fene, bexc, stack), vir[6]. */
void oxo_bonded(const oxg_bonded_params* p, const double Rc[3], const double qA[4],
                const double qB[4], int typeA, int typeB, double FB[3], double tauA[3],
                double tauB[3], double e[3], double vir[6]);

/* ---- system driver ------------------------------------------------------------ */
typedef struct oxo_model {
    int n_types;
    int n_bond_types;
    /* per term: n_types*n_types params (row-major [ti][tj]) + r_cut; have[t] != 0
     * when the term's parameters are present. */
    const oxg_excvol_params* excvol;
    const oxg_hbond_params* hbond;
    const oxg_cross_params* cross;
    const oxg_hbondcross_params* hbondcross;
    const oxg_coax_params* coax;
    const oxg_debye_params* debye;
    const double* r_cut[OXG_N_PAIR_TERMS];
    const oxg_bonded_params* bonded; /* n_bond_types entries */
} oxo_model;

typedef struct oxo_system {
    int N;
    const double* pos;    /* 3*N */
    const double* quat;   /* 4*N (w,x,y,z) */
    const int32_t* type;  /* N */
    const double* charge; /* N (may be NULL: all 1) */
    double box[3];
    int n_bonds;
    const int32_t* bonds; /* 3*n_bonds: A, B, bond_type */
} oxo_system;

/* Forces of the selected terms at the given state. Outputs (any may be NULL):
 * force[4N] (x,y,z, per-particle energy), torque[3N], pair_energy[6], bonded_energy[3],
 * pair_count[6] (pairs with rsq < rcutsq per term), virial[6] (bonded site virial sum).
 * Uses an O(N^2) pair loop when use_cells == 0, else a cell list. Returns 0. */
int oxo_forces(const oxo_model* m, const oxo_system* s, uint32_t term_mask, int bonded,
               int use_cells, double* force, double* torque, double* pair_energy,
               double* bonded_energy, int64_t* pair_count);

/* Langevin MD (velocity Verlet + Miller NO_SQUISH rotation + Langevin bath) in FP64
 * with the same counter-based RNG as the GPU engine. State arrays are updated in
 * place: pos[3N], quat[4N], vel[3N], angmom[4N]. Unit mass and inertia. Uses a
 * Verlet list of radius max(r_cut)+buffer, rebuilt when a particle moved more than
 * buffer/2 (HOOMD Cell nlist semantics). n_threads > 1 uses OpenMP.
 * Returns the number of neighbour-list builds, or -1 on error. */
long oxo_langevin_run(const oxo_model* m, oxo_system* s, double* pos, double* quat,
                      double* vel, double* angmom, uint32_t term_mask, int bonded,
                      double dt, double kT, double gamma, double gamma_r, uint64_t seed,
                      long step0, long nsteps, double buffer, int n_threads);

/* Counter-based RNG shared with the GPU engine (Philox4x32-10, Salmon et al. 2011). */
void oxo_philox4x32(uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

#ifdef __cplusplus
}
#endif
#endif
