/*
 * bmxg.h -- C ABI of the GB300-native BMX particle DEM step.
 *
 * This library replaces the particle step that the reference performs in
 *   BMXParticleContainer::EvolveParticles(dt, cost, knapsack_weight_type, nsubsteps)
 *   (src/des/bmx_pc.H:126-129, implementation src/des/bmx_pc_interaction.cpp:13-495)
 * i.e. the cell-binned neighbour search (AMReX buildNeighborList with
 * BMXCheckPair, src/des/bmx_pc.H:55-82), the force gather over the full
 * neighbour list (bmx_pc_interaction.cpp:170-279) with the force laws of
 * src/chemistry/bmx_cell_interaction_K.H, and the overdamped update
 * (bmx_pc_interaction.cpp:311-449), followed by the periodic wrap that the
 * trailing Redistribute applies (bmx_pc_interaction.cpp:485-486).
 *
 * Conventions
 *  - Every entry point returns an int status (BMXG_OK == 0, negative on error)
 *    and never throws or exits; bmxg_last_error() gives a one-line message.
 *  - A context is used by one host thread at a time (the reference has one
 *    caller thread, src/timestepping/bmx_evolve.cpp:97).
 *  - Particle arrays are structure-of-arrays with one entry per particle; the
 *    field names are the reference's realIdx / intIdx names
 *    (src/chemistry/bmx_chem.H:38-118).  Pointers are host pointers unless
 *    the call takes `where == BMXG_DEVICE`.
 *  - No torch types cross this boundary.
 */
#ifndef BMXG_H
#define BMXG_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BMXG_ABI_VERSION 2

/* status codes */
#define BMXG_OK              0
#define BMXG_ERR_ARG        -1  /* bad argument (NULL, n < 0, bad geometry)      */
#define BMXG_ERR_CUDA       -2  /* a CUDA runtime call failed                    */
#define BMXG_ERR_OOM        -3  /* device allocation failed                      */
#define BMXG_ERR_CAPACITY   -4  /* caller buffer too small (pair list export)    */
#define BMXG_ERR_STATE      -5  /* call out of order (e.g. step before set_state) */
#define BMXG_ERR_NONFINITE  -6  /* a non-finite position/velocity was produced   */
#define BMXG_ERR_TIMEOUT    -7  /* a device-side wait ran out of its budget      */
#define BMXG_ERR_UNSUPPORTED -8 /* configuration outside what this build covers  */

/* where the particle arrays live */
#define BMXG_HOST   0
#define BMXG_DEVICE 1

/* arithmetic form of the pair math */
#define BMXG_FP64   0  /* plain form: FP64 throughout (reference arithmetic)        */
#define BMXG_FP32F  1  /* precision form: FP32 pair math on FP64-differenced
                          bin-relative offsets, FP64 positions and closest-point
                          solve of near-parallel segments                            */

/* cell types (cellType, src/chemistry/bmx_chem.H:120-126) */
#define BMXG_YEAST 0
#define BMXG_FUNGI 1

/* siteLocation (src/chemistry/bmx_chem.H:128-136) */
#define BMXG_SITE_TIP      0
#define BMXG_SITE_SECOND_1 1
#define BMXG_SITE_SECOND_2 2
#define BMXG_SITE_INTERIOR 3

/*
 * Force parameters.  The first nine fields are, in order, the vector that
 * BMXCellInteraction::getForceParams() returns (fpar[0..8],
 * src/chemistry/bmx_cell_interaction.cpp:84-93), read from the deck keys
 * cell_force.{boundary_width, stiffness, wall_boundary_width, wall_stiffness,
 * gravity, bond_strength, bond_cutoff, viscous_drag} and fluid.surface_location.
 */
typedef struct bmxg_params {
    double bndry_width;    /* fpar[0] adhesion band width of the cubic law       */
    double stiffness;      /* fpar[1] cell-cell stiffness (drag folded in)       */
    double z_wall;         /* fpar[2] growth-surface location                    */
    double z_bndry_width;  /* fpar[3] wall adhesion band width                   */
    double z_stiffness;    /* fpar[4] wall stiffness                             */
    double z_gravity;      /* fpar[5] gravity factor                             */
    double bond_strength;  /* fpar[6] harmonic bond strength (rods)              */
    double bond_cutoff;    /* fpar[7] (carried; unused by the step)              */
    double viscosity;      /* fpar[8] viscous drag of rod segments               */
    /* DEM::neighborhood (src/chemistry/bmx_chem.cpp:124).  BMXCheckPair
     * compares it with the SQUARED centre distance (src/des/bmx_pc.H:72,76),
     * exactly as the reference does.                                          */
    double neighborhood;
} bmxg_params;

/*
 * Geometry of one colony (one AMReX level geometry).  Bins are the level's
 * cells: dx = (prob_hi - prob_lo) / n_cell, dxi = 1 / dx.  x and y may be
 * periodic (n_cell >= 3 there); z must be non-periodic (the growth surface
 * sits in z, src/chemistry/bmx_cell_interaction_K.H:1005-1283).
 */
typedef struct bmxg_geometry {
    double  prob_lo[3];
    double  prob_hi[3];
    int32_t n_cell[3];
    int32_t is_periodic[3];
} bmxg_geometry;

/*
 * Particle state, SoA.  A NULL pointer means "not supplied" on input and
 * "not wanted" on output.  Arrays marked [4] hold four planes of n entries
 * (entry k of particle i at [k*n + i]), mirroring seg1..seg4 in intIdx.
 * Spheres (all cell_type == YEAST) need x, y, z, radius, cell_type only.
 */
typedef struct bmxg_particles {
    int64_t n;
    /* positions */
    double *x, *y, *z;
    /* realIdx fields read by the step */
    double *radius, *c_length, *theta, *phi, *area, *bond_scale;
    /* realIdx fields written by the step (velx..velz = fc[0..2], wx..wz = fc[3..5]) */
    double *velx, *vely, *velz, *wx, *wy, *wz;
    /* intIdx fields */
    int32_t *cell_type;
    int32_t *id, *cpu;
    int32_t *n_bnds;
    int32_t *seg_id1;   /* [4] seg1_id1 .. seg4_id1 */
    int32_t *seg_id2;   /* [4] seg1_id2 .. seg4_id2 */
    int32_t *site;      /* [4] site1 .. site4       */
    int32_t *position;
    int32_t *fuse_tip;
    int32_t *fix_site;
    int32_t *fuse_flag, *split_flag, *new_flag;
    int32_t *dltd;      /* [6] dltd_site1, dltd_site2, dltd_id1, dltd_id2, dltd_cpu1, dltd_cpu2 */
} bmxg_particles;

/* counters of the last bmxg_step call */
typedef struct bmxg_stats {
    int64_t n_particles;
    int64_t n_pairs_last;       /* neighbour-list entries of the last step        */
    int64_t n_out_of_domain;    /* particles outside the non-periodic z range     */
    int64_t n_edge_ghost;       /* periodic images whose bin left the halo cell   */
    int64_t n_bond_repairs;     /* half-bonds repaired (rods)                      */
    int64_t n_rebins;           /* bin-order rebuilds: one per step, or one per
                                   list build in the FP32F list mode (cumulative) */
    int64_t n_kernel_launches;  /* kernels this context enqueued, graph nodes counted */
    int64_t main_kernel_launches; /* force-kernel launches timed while profiling     */
    double  main_kernel_ms;     /* their summed device time (profiling mode)        */
    double  last_step_ms;       /* device time of the last bmxg_step call          */
} bmxg_stats;

typedef struct bmxg_ctx bmxg_ctx;

/* ---- lifetime ---------------------------------------------------------- */

/* Create a context for `ncolonies` independent colonies (1 for the plain
 * single-domain step).  geoms[ncolonies].  Replaces the construction of
 * BMXParticleContainer (src/des/bmx_pc.cpp:17-41) and
 * BMXCellInteraction::setParams (src/chemistry/bmx_cell_interaction.cpp:54-95). */
int  bmxg_create(const bmxg_params *params, int32_t ncolonies,
                 const bmxg_geometry *geoms, bmxg_ctx **out);
void bmxg_destroy(bmxg_ctx *ctx);
const char *bmxg_last_error(const bmxg_ctx *ctx);
int  bmxg_version(void);

/* Replace the force parameters (fpar) between steps. */
int  bmxg_set_params(bmxg_ctx *ctx, const bmxg_params *params);

/* Set the CUDA stream (a cudaStream_t passed as void*) all work goes to.
 * NULL selects the context's own stream. */
int  bmxg_set_stream(bmxg_ctx *ctx, void *stream);

/* ---- state ------------------------------------------------------------- */

/* Load particles.  colony_offsets[ncolonies+1] gives each colony's particle
 * range (NULL when ncolonies == 1).  Replaces InitParticlesAscii + the
 * Redistribute that follows (src/des/bmx_pc_init.cpp:17-132). */
int  bmxg_set_state(bmxg_ctx *ctx, const bmxg_particles *p,
                    const int64_t *colony_offsets, int where);

/* Read particles back in the caller's original order.  Only non-NULL
 * arrays are written. */
int  bmxg_get_state(bmxg_ctx *ctx, bmxg_particles *p, int where);

/* ---- the step ---------------------------------------------------------- */

/* Advance `nsteps` DEM steps of size dt.  One step is one call of
 * EvolveParticles with nsubsteps == 1 (bmx_pc_interaction.cpp:56-65 always
 * yields one substep): neighbour rebuild, force gather + wall force, update,
 * periodic wrap.  `precision` is BMXG_FP64 or BMXG_FP32F.  The step loop is
 * replayed from a captured CUDA graph. */
int  bmxg_step(bmxg_ctx *ctx, double dt, int32_t nsteps, int32_t precision);

/* Instantiate, without running a step, the CUDA graphs that bmxg_step(ctx, dt,
 * n, precision) replays (the graph of the re-sync period and the one-step
 * graphs, from either parity) and allocate the buffers of that path, so that
 * the first long call captures nothing.  The FP32F list path counts as chosen
 * (a later one-step call then steps over the list too).  No counterpart in the
 * reference (it has no graphs). */
int  bmxg_prepare(bmxg_ctx *ctx, double dt, int32_t precision);

/* Drop-in for the reference member function, on the state loaded with
 * bmxg_set_state: nsubsteps is written (always 1), cost_per_colony (may be
 * NULL) receives the particle count per colony as the "NumParticles" cost
 * (bmx_pc_interaction.cpp:460-475). */
int  bmxg_evolve_particles(bmxg_ctx *ctx, double dt, double *cost_per_colony,
                           int32_t *nsubsteps);

/* The same step on particles kept in the reference's own layout:
 * amrex::Particle<nreal, nint> of AMReX 22.x in double precision, i.e.
 * double pos[3]; double rdata[nreal]; int id, cpu; int idata[nint]
 * (448-byte structs for BMX's 34 / 35, src/chemistry/bmx_chem.H:16-17), in
 * host memory.  Loads them, runs one step (bmxg_evolve_particles) and writes
 * back what EvolveParticles writes: pos, velx..velz, wx..wz, theta, phi and
 * the integer fields its pair loop and wall force change
 * (bmx_pc_interaction.cpp:174-279, :317-436).  nreal >= 25, nint >= 35. */
int  bmxg_evolve_particles_aos(bmxg_ctx *ctx, void *particles, int64_t n,
                               int32_t nreal, int32_t nint,
                               const int64_t *colony_offsets, double dt,
                               double *cost_per_colony, int32_t *nsubsteps);

int  bmxg_get_stats(const bmxg_ctx *ctx, bmxg_stats *out);

/* Profiling mode: when on, bmxg_step launches eagerly (no graph) and times
 * the force kernel of every step with CUDA events on the context's stream;
 * the sums land in bmxg_stats.main_kernel_ms / main_kernel_launches.
 * Turning it on resets those sums. */
int  bmxg_set_profiling(bmxg_ctx *ctx, int32_t on);

/* ---- neighbour list export ---------------------------------------------- */

/* Neighbour list of the CURRENT state, built exactly as the step builds it:
 * for particle i (original order) entries offs[i]..offs[i+1]-1 of idx/img.
 * idx = original index of the neighbour's source particle; img = periodic
 * image code (sx+1) + 3*(sy+1), 4 meaning "no shift".  offs has n+1 entries.
 * Returns BMXG_ERR_CAPACITY (and *total) if cap is too small.  Replaces
 * m_neighbor_list[lev][index] of AMReX buildNeighborList
 * (bmx_pc_interaction.cpp:103,155,185-189). */
int  bmxg_get_pairs(bmxg_ctx *ctx, int64_t *offs, int32_t *idx, int8_t *img,
                    int64_t cap, int64_t *total);

/* ---- differentiation form ------------------------------------------------ */

/* Contact-parameter extensions of the sphere law used by the differentiable
 * step (all zero: the reference law, bit for bit):
 *   damping   gamma of a two-body overdamped dashpot, F -> F / (1 + gamma (m_i + m_j))
 *   mu        Stokes drag: pair forces move sphere i with mobility
 *             m_i = 1 / (6 pi mu r_i) instead of 1 (the reference folds drag into k)
 *   adhesion  per-particle adhesion energy a_i (caller order, NULL = 0) in units
 *             of the band's spring energy: F -= k bw (a_i + a_j)/2 (r - rA)^2
 * Set after bmxg_set_state (the adhesion array follows the loaded state). */
typedef struct bmxg_ext {
    double damping;
    double mu;
    const double *adhesion;
} bmxg_ext;
int  bmxg_set_ext(bmxg_ctx *ctx, const bmxg_ext *ext);

/* Differentiable FP64 trajectory of nsteps spheres steps from the loaded
 * state (the loaded state then holds the final positions), keeping a
 * checkpoint of the positions every ckpt_every steps. */
int  bmxg_forward(bmxg_ctx *ctx, double dt, int32_t nsteps, int32_t ckpt_every);

/* Hand-written adjoint of that trajectory.  dL_dx: [3][n] gradient of a loss
 * with respect to the final positions (x plane, y plane, z plane; caller
 * order).  Out (each may be NULL): dL_dx0 [3][n] gradient with respect to the
 * initial positions, dL_dparams[3] = dL/d(stiffness, damping, mu),
 * dL_dadhesion [n].  Segments between checkpoints are recomputed forward and
 * swept backward; the neighbour lists are the ones the forward step built. */
int  bmxg_backward(bmxg_ctx *ctx, const double *dL_dx, double *dL_dx0,
                   double *dL_dparams, double *dL_dadhesion);

/* ---- a step that allocates nothing ---------------------------------------- */

/* One FP64 step of a sphere colony on caller-owned DEVICE arrays, without
 * any device allocation.  This entry point has no counterpart in the
 * reference; it exists for callers that may not call cudaMalloc on the
 * step's path: an application that hands out all device memory through its
 * own arenas, sized up front (as AMReX does), where a library allocating
 * behind the arena can make the arena's next allocation fail.
 * Inputs x, y, z, radius (n each) and outputs x_out, y_out, z_out and
 * vel_x..vel_z (n each; may not alias the inputs) are device pointers in
 * the caller's order; all particles are spheres of one colony with geometry
 * `geom`.  The result equals bmxg_set_state + bmxg_step(dt, 1, BMXG_FP64) +
 * bmxg_get_state bit for bit.
 * Limits: n <= 32768 and n_cell[0] * n_cell[1] <= 65536, else
 * BMXG_ERR_CAPACITY.  The binning scratch is one fixed device array of about
 * 2.4 MB that every GPU loading the library holds until the process exits.
 * The first call on a device looks up that array's address.  Every call
 * reuses the array: calls that
 * overlap on the GPU (other streams, other host threads) race and must not
 * be issued.
 * Runs on `stream` (a cudaStream_t; NULL = the legacy default stream) and
 * returns after it completes.  *n_out_of_domain (may be NULL) receives the
 * particles whose new z left the non-periodic range (kept, as bmxg_step
 * keeps them and counts them in bmxg_stats.n_out_of_domain).  Returns
 * BMXG_ERR_NONFINITE for a non-finite new position and BMXG_ERR_STATE when
 * the counting sort's counts came out inconsistent (an internal error), as
 * bmxg_step does. */
int  bmxg_sphere_step_noalloc(const bmxg_params *params, const bmxg_geometry *geom,
                              int64_t n, const double *x, const double *y,
                              const double *z, const double *radius,
                              double *x_out, double *y_out, double *z_out,
                              double *vel_x, double *vel_y, double *vel_z,
                              double dt, void *stream, int64_t *n_out_of_domain);

/* ---- start-up bonds ----------------------------------------------------- */

/* InitBonds on the CURRENT state: for every FUNGI-FUNGI pair of the step's
 * neighbour list within the interaction gate, the first of the end pairs
 * (site1,site1), (site2,site1), (site1,site2), (site2,site2) closer than rlim
 * appends (id, cpu of the neighbour, site of the segment) to the segment's
 * own bond table.  rlim <= 0 selects the reference's 1e-7.  Replaces
 * BMXParticleContainer::InitBonds (src/des/bmx_pc_interaction.cpp:500-668,
 * with fixBonds of src/chemistry/bmx_cell_interaction_K.H:1287-1440), which
 * src/timestepping/bmx_evolve.cpp:95 calls once at time 0.  The neighbour's
 * side is written to a copy in the reference and discarded, as here.
 * *added / *overflow (may be NULL) receive the bonds appended and those that
 * found the table full; the reference writes the latter past its four slots,
 * here they are dropped and the call returns BMXG_ERR_CAPACITY. */
int  bmxg_init_bonds(bmxg_ctx *ctx, double rlim, int64_t *added, int64_t *overflow);

/* ---- species exchange between bonded segments ---------------------------- */

/* One substep of BMXParticleContainer::ParticleExchange
 * (src/des/bmx_pc_xchng.cpp:13-257, with initExchange / evaluateExchange /
 * applyIncrements of src/chemistry/bmx_chem_K.H:1949-2126) on the CURRENT
 * state and its neighbour list: each FUNGI segment exchanges species A, B, C
 * with every listed FUNGI neighbour that both hold in their bond tables,
 * d = (c_i - c_j) * pi (r_i^2 + r_j^2) / 2 * mt * dt, clamped as the
 * reference clamps it, and adds -d / vol_i.  conc: 3 planes of n (A, B, C;
 * caller order), updated in place; vol: n; xpar = {mass_transfer_A, _B, _C}
 * (BMXChemistry::getExchangeParameters, src/chemistry/bmx_chem.cpp:221-228).
 * where: BMXG_HOST or BMXG_DEVICE for conc and vol (xpar is a host array).  The reference keeps the
 * concentrations in the particles' real data (realIdx::first_data + 0..2);
 * here they are the caller's arrays. */
int  bmxg_particle_exchange(bmxg_ctx *ctx, const double *vol, double *conc, double dt,
                            const double xpar[3], int32_t where);

/* ---- cell division ------------------------------------------------------- */

/* Parameters of the division step (SPECIES::max_vol, max_seg_length,
 * max_seg_radius, branching_probability, split_probability, seg_split_length
 * of src/mods/bmx_chem_species_parms.cpp:55-70; BMXChemistry::p_overlap,
 * p_num_reals, p_num_ints of src/chemistry/bmx_chem.cpp:29-53,110). */
typedef struct bmxg_split_params {
    double  max_vol;     /* a YEAST cell with vol > max_vol divides                       */
    double  overlap;     /* p_overlap (0.2): mother and daughter overlap by this fraction */
    double  max_len;     /* a FUNGI tip at least this long ...                            */
    double  max_rad;     /* ... and at least this wide splits                             */
    double  brnch_prob;  /* a segment behind a tip branches with this probability         */
    double  split_prob;  /* a splitting tip with bonds splits in two with 1 - this        */
    double  split_len;   /* length a splitting tip keeps                                  */
    int32_t num_reals;   /* p_num_reals (3 x species): reals copied past first_data        */
    int32_t num_ints;    /* p_num_ints (0): ints copied past first_data                    */
} bmxg_split_params;

/* BMXParticleContainer::split_particles (src/des/bmx_split_particles.cpp:16-166,
 * with checkSplit, copyChildParameters, setNewCell, setNewSegment and
 * setNewSegments of src/chemistry/bmx_chem_K.H:23-69,357-1011,2129-2494) on
 * particles in the reference's own layout (the AoS records of
 * bmxg_evolve_particles_aos, nreal >= 34, nint >= 35):
 *  - a YEAST cell with vol > max_vol divides in two along a random direction;
 *  - a FUNGI tip with radius >= max_rad and c_length >= max_len either grows a
 *    new tip (or halves, when it has no bonds) or, with probability
 *    1 - split_prob, splits into two tips;
 *  - a FUNGI segment right behind a tip grows a side branch with probability
 *    brnch_prob.
 * New particles are appended at particles[n + k], k counting the new particles
 * before them in array order (the reference's exclusive scan; a two-way split
 * appends two), with id next_id + k and cpu my_proc.
 * Random draws: `draws` (ndraws values in [0, 1)) is the sequence a serial run
 * of the reference takes from amrex::Random, in its order: one per FUNGI tip
 * at the radius limit and per segment behind a tip (checkSplit, array order),
 * then per division in array order 2 (YEAST cell), 2 (new tip), 3 (side
 * branch), 4 (two-way split) or 0 (isolated segment).  With draws == NULL a
 * SplitMix64 counter generator keyed by seed and the cell's id and cpu
 * supplies them, the same on every device and host.  Fields the reference
 * leaves unset in a new particle are not written.
 * *num_split receives the number of new particles.  When n + *num_split > cap,
 * or draws holds fewer values than the call takes, the call returns
 * BMXG_ERR_CAPACITY or BMXG_ERR_ARG and writes nothing else.  where:
 * BMXG_HOST (particles and draws in host memory) or BMXG_DEVICE (device
 * memory).  Runs on `stream` (NULL = legacy default stream) and returns after
 * it completes; the host reads the totals in between, as the reference does
 * (bmx_split_particles.cpp:58-66).  Each device keeps a scratch of about 17
 * bytes per particle of the largest call so far (and 32 bytes of pinned host
 * memory) until the process exits; calls on one device run one at a time.
 * Host-memory calls also stage the records on the device for the call. */
int  bmxg_split_cells_aos(const bmxg_split_params *sp, void *particles, int64_t n, int64_t cap,
                          int32_t nreal, int32_t nint, const double *draws, int64_t ndraws,
                          uint64_t seed, int64_t next_id, int32_t my_proc, int32_t where,
                          int64_t *num_split, void *stream);

/* ---- fixture I/O (host only; no context, no device) ---------------------- */

/* Particle input file of BMXParticleContainer::InitParticlesAscii
 * (src/des/bmx_pc_init.cpp:17-132): the count, then 27 values per particle
 * (x y z radius c_length theta phi area vol velx vely velz wx wy wz fx fy fz
 * taux tauy tauz gx gy gz dadt dvdt cell_type), read as one stream.  Fields
 * the file does not carry get the reference's values (id = 1..n, cpu = 0,
 * bond_scale = 1, no bonds).  Call with out == NULL (or cap too small) to
 * get the count in *n (BMXG_ERR_CAPACITY); then with out->n == *n.  Only the
 * non-NULL arrays of out are filled. */
int  bmxg_read_ascii(const char *path, bmxg_particles *out, int64_t cap, int64_t *n);

/* The same format written from a state (vol from the shape; force, torque,
 * gradient and rates as 0), 17 significant digits: bmxg_read_ascii reads
 * back the same doubles.  The reference has no writer for this format. */
int  bmxg_write_ascii(const char *path, const bmxg_particles *p);

/* Legacy-VTK polydata of BMXParticleContainer::WriteToAscii
 * (src/des/bmx_pc_write.cpp:11-219): segment end points pos +- L/2 n, one
 * polygon per particle, the particle index as scalar and conc_b (may be
 * NULL: 0) as the "conc_B" scalar of both end points. */
int  bmxg_write_vtk(const char *path, const bmxg_particles *p, const double *conc_b);

/* Particles of an AMReX checkpoint in the Version_Two_Dot_One_double format
 * (dir = .../chkNNNNN/particles; written by bmx::WriteCheckPointFile,
 * src/io/bmx_chk.cpp:114-160, read back by bmx::Restart,
 * src/io/bmx_restart.cpp:24-225), all grids of `level` (-1: every level).
 * Component layouts: the current realIdx/intIdx (34 real, 35 int) and the
 * 33 + 33 layout of the checkpoints shipped in exec/ (realIdx without
 * bond_scale, intIdx without fuse_tip and fix_site; those get 1 and 0).
 * Two-call protocol as bmxg_read_ascii. */
int  bmxg_read_checkpoint(const char *dir, int32_t level, bmxg_particles *out, int64_t cap, int64_t *n);

/* Message of the last failed fixture I/O call of this thread. */
const char *bmxg_io_last_error(void);

/* Gated pairs of the LAST FP32F list step, as that step accumulated them:
 * with capture on (bmxg_set_pair_capture), every list step records, per
 * particle, the neighbours whose pair passed the force gate r^2 < rA^2
 * (bmx_pc_interaction.cpp:212) in the order the step summed them.  For
 * particle i (original order) entries offs[i]..offs[i+1]-1 of idx hold the
 * original indices of those neighbours (offs: n+1 entries; idx may be NULL
 * for the counts only).  Returns BMXG_ERR_STATE when the last step was not a
 * list step recorded with capture on, BMXG_ERR_CAPACITY (and *total) when
 * cap is too small or a particle had more than 32 gated pairs.  A check of
 * the list the step walks against the reference's gated pair set; it has no
 * counterpart in the reference (AMReX's list holds every stencil pair and the
 * gate runs inside the force loop). */
int  bmxg_set_pair_capture(bmxg_ctx *ctx, int32_t on);
int  bmxg_get_step_pairs(bmxg_ctx *ctx, int64_t *offs, int32_t *idx, int64_t cap, int64_t *total);

/* ---- tuning ------------------------------------------------------------- */

/* FP32F sphere steps keep a neighbour list with a skin between builds when it
 * reproduces the reference's pair set exactly: the largest force cutoff
 * 2 r_max + bndry_width plus the skin fits inside the smallest bin width, and
 * BMXCheckPair holds for every stencil pair.  mode 1 (default) uses it there,
 * mode 0 never (every step re-bins and walks the stencil).  The reference
 * rebuilds its AMReX neighbour list every step (bmx_pc_interaction.cpp:97-103);
 * this switch has no counterpart there. */
int  bmxg_set_list_mode(bmxg_ctx *ctx, int32_t mode);

/* Time the launch shapes of the step kernels on the loaded state and keep
 * the fastest: the per-step stencil kernels of both forms (block, grid) and,
 * where the FP32F list path applies, the list step (block, passes of the
 * block per chunk of slots) and the list build (block).  Results are cached
 * in a JSON file at cache_path (may be NULL: no cache), keyed by the device,
 * the particle count and the colony-size histogram.  The loaded state is left
 * as it was.  The reference has no counterpart (AMReX tiles its loops by a
 * fixed tile size, bmx_pc_interaction.cpp:111-114). */
int  bmxg_autotune(bmxg_ctx *ctx, const char *cache_path);

/* ---- one tile with the caller's ghost particles ------------------------- */

/* A tile of the level's domain (the context's one geometry): its first and
 * last cell per axis, 0-based and inclusive (an AMReX Box). */
typedef struct bmxg_tile {
    int32_t lo[3];
    int32_t hi[3];
} bmxg_tile;

/* One FP64 step of the spheres (YEAST) of one tile: AMReX's per-tile
 * EvolveParticles (src/des/bmx_pc_interaction.cpp:97-279) after fillNeighbors
 * has put the particles within one cell of the tile beside its own -- the
 * ghosts, periodic images already shifted by a domain length (the halo of
 * src/des/bmx_pc.cpp:23).  reals: x, y, z, radius, cell_type in; x, y, z
 * replaced by the new positions (periodically wrapped, as the trailing
 * Redistribute does) and velx, vely, velz written.  ghosts (NULL or n = 0:
 * none): x, y, z, radius, cell_type, read only.  The neighbour list holds the
 * reals and the ghosts in the order of the whole-domain step (cells x, y, z;
 * within a cell the reals in the caller's order, then the ghosts in theirs),
 * so that tiles covering the domain, each with the ghosts the whole-domain
 * step would see, give the whole-domain step's results bit for bit.  The
 * context needs no loaded state; its one geometry is the level's domain.
 * where: BMXG_HOST or BMXG_DEVICE for every array.  Returns BMXG_ERR_ARG when
 * a real particle is outside the tile or a ghost outside its one-cell halo,
 * BMXG_ERR_UNSUPPORTED for a particle that is not YEAST (rod segments need
 * their neighbours' bond tables: a whole-domain step), BMXG_ERR_NONFINITE
 * (after writing the results) when a new position is not finite. */
int  bmxg_step_tile(bmxg_ctx *ctx, const bmxg_tile *tile, const bmxg_particles *reals,
                    const bmxg_particles *ghosts, double dt, int32_t where);

/* The launch shapes in use (defaults until bmxg_autotune picks others). */
typedef struct bmxg_shapes {
    int32_t sphere_block[2];    /* per-step stencil kernel, [FP64, FP32F]            */
    int32_t sphere_grid[2];     /* 0: one slot per thread                            */
    int32_t list_step_block;    /* FP32F list step                                   */
    int32_t list_step_passes;   /* passes of the block per chunk (0: the size rule)  */
    int32_t list_build_block;   /* list build                                        */
    int32_t list_step_persistent; /* 1: one wave of blocks taking chunks from a counter */
} bmxg_shapes;
int  bmxg_get_shapes(const bmxg_ctx *ctx, bmxg_shapes *out);
/* Use these shapes (blocks a multiple of 32 up to 256, grid >= 0, passes
 * 0..64; else BMXG_ERR_ARG): pins what bmxg_autotune would pick.  The results
 * of a step do not depend on the shapes. */
int  bmxg_set_shapes(bmxg_ctx *ctx, const bmxg_shapes *in);

#ifdef __cplusplus
}
#endif
#endif /* BMXG_H */
