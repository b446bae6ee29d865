/*
 * bmx_oracle.h -- CPU oracle of the BMX particle DEM step.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (boltzmannmfx_gb300/,
 * include/) links or calls this code; tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py use it as the checker.
 *
 * It is a plain-C restatement of the reference path:
 *   - neighbour list: AMReX NeighborParticleContainer::buildNeighborList with
 *     BMXCheckPair(DEM::neighborhood, false) (src/des/bmx_pc.H:55-82,
 *     src/des/bmx_pc_interaction.cpp:97-103), periodic ghosts of fillNeighbors
 *     with a one-cell halo (src/des/bmx_pc.cpp:23).  AMReX itself is not in the
 *     reference tree, so this part is a behavioural restatement: PARITY
 *     UNPINNED for the pair-list construction and the periodic wrap.
 *   - force gather + wall force: src/des/bmx_pc_interaction.cpp:170-279 with
 *     the force laws of src/chemistry/bmx_cell_interaction_K.H.
 *   - update: src/des/bmx_pc_interaction.cpp:311-449.
 * The force gather and update are pinned against the reference's own code:
 * oracle/ref_harness.cpp compiles bmx_cell_interaction_K.H and the two loop
 * bodies of bmx_pc_interaction.cpp verbatim (oracle/Makefile), and
 * tests/golden/ holds vectors produced by it.
 */
#ifndef BMX_ORACLE_H
#define BMX_ORACLE_H
#include "../include/bmxg.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Neighbour list of one colony, restating AMReX buildNeighborList. */
int  orc_pairs(const bmxg_params *prm, const bmxg_geometry *geom,
               const bmxg_particles *p, int64_t *offs, int32_t *idx,
               int8_t *img, int64_t cap, int64_t *total);

/* Force gather + wall force over a given list (bmx_pc_interaction.cpp:170-279).
 * fc is 6*n planar (fc[c*n+i]).  Applies the step's integer side effects
 * (flag resets, rod half-bond repair, dltd reset, position fix, fix_site). */
int  orc_forces(const bmxg_params *prm, const bmxg_geometry *geom,
                bmxg_particles *p, const int64_t *offs, const int32_t *idx,
                const int8_t *img, double *fc, int nthreads);

/* Update (bmx_pc_interaction.cpp:311-436) followed by the periodic wrap of
 * the trailing Redistribute. */
void orc_update(const bmxg_geometry *geom, bmxg_particles *p, const double *fc,
                double dt, int nthreads);

/* Periodic wrap alone (AMReX enforcePeriodic restated). */
void orc_wrap(const bmxg_geometry *geom, bmxg_particles *p);

/* Full step loop over `ncol` colonies (offsets[ncol+1], NULL when ncol==1). */
int  orc_evolve(const bmxg_params *prm, int32_t ncol, const bmxg_geometry *geoms,
                const int64_t *offsets, bmxg_particles *p, double dt,
                int32_t nsteps, int nthreads);

/* Sample-and-time helper for the CPU baseline: runs orc_evolve and returns
 * the wall-clock seconds. */
double orc_time_evolve(const bmxg_params *prm, int32_t ncol,
                       const bmxg_geometry *geoms, const int64_t *offsets,
                       bmxg_particles *p, double dt, int32_t nsteps,
                       int nthreads);

/* InitBonds: bond segments whose ends are closer than rlim (1e-7 in the
 * reference, bmx_pc_interaction.cpp:508), over the given neighbour list. */
int  orc_init_bonds(const bmxg_params *prm, const bmxg_geometry *geom, bmxg_particles *p,
                    const int64_t *offs, const int32_t *idx, const int8_t *img, double rlim,
                    int64_t *added, int64_t *overflow);

/* ParticleExchange over the given neighbour list (bmx_pc_xchng.cpp:13-257,
 * bmx_chem_K.H:1949-2126): conc 3 planes (A, B, C) updated in place, vol per
 * particle, xpar = {mass_transfer_A, _B, _C}. */
int  orc_particle_exchange(const bmxg_geometry *geom, const bmxg_particles *p, const int64_t *offs,
                           const int32_t *idx, const double *vol, double *conc, double dt,
                           const double xpar[3]);

/* split_particles (bmx_split_particles.cpp:16-166, checkSplit /
 * copyChildParameters / setNewCell / setNewSegment / setNewSegments of
 * bmx_chem_K.H:23-69,357-1011,2129-2494) on AoS records, with the contract of
 * bmxg_split_cells_aos (host memory). */
int  orc_split_cells_aos(const bmxg_split_params *sp, void *particles, int64_t n, int64_t cap,
                         int32_t nreal, int32_t nint, const double *draws, int64_t ndraws,
                         uint64_t seed, int64_t next_id, int32_t my_proc, int64_t *num_split);
double orc_split_uniform(uint64_t seed, int32_t id, int32_t cpu, int32_t j);

/* Single-pair / single-particle entry points used by unit tests. */
void orc_pair_force(const bmxg_params *prm, const double r12[3],
                    const bmxg_particles *p, int64_t i, int64_t j,
                    double v1[3], double rot1[3]);
void orc_surface_force(const bmxg_params *prm, const bmxg_particles *p,
                       int64_t i, double vel[3], double rot[3]);
void orc_min_distance(const double e[12], double *tau_i, double *tau_j);

#ifdef __cplusplus
}
#endif
#endif
