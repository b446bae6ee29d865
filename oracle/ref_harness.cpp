// ref_harness.cpp -- the reference's own step code, compiled on the host.
//
// TEST INFRASTRUCTURE ONLY (builds oracle/_ref/libbmxref.so, which the
// golden-vector script and the oracle tests load; the product never does).
//
// What is the reference's code here, compiled verbatim:
//   * src/chemistry/bmx_cell_interaction_K.H (maxInteractionDistance,
//     evaluateMinimumDistance, evaluateForce, evaluateSurfaceForce), included
//     from the reference tree through the stand-in AMReX headers in shim/;
//   * the body of the force-gather lambda, src/des/bmx_pc_interaction.cpp:174-278
//   * the body of the update lambda,       src/des/bmx_pc_interaction.cpp:317-436
//   * the body of the InitBonds lambda,    src/des/bmx_pc_interaction.cpp:577-626
//   * the body of the exchange lambda,     src/des/bmx_pc_xchng.cpp:122-151, with
//     initExchange / evaluateExchange / applyIncrements of
//     src/chemistry/bmx_chem_K.H (included verbatim)
//     (cut out of the reference file by oracle/Makefile into _ref/ and
//     #included below inside plain loops over i, i.e. the serial CPU build).
// What is NOT the reference's code: the neighbour list and the periodic wrap
// (AMReX, absent from the reference tree) come from the oracle port
// (bmx_oracle.c), and the small stand-in types below replace amrex::Particle,
// RealVect, the neighbour iterator and Gpu::Atomic::Add.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <vector>

#include <bmx_cell_interaction_K.H>
#include <bmx_chem_K.H>

#include "bmx_oracle.h"

namespace amrex { namespace Gpu { namespace Atomic {
inline void Add(double *p, double v) { *p += v; }
} } }
#define AMREX_ASSERT_WITH_MESSAGE(cond, msg) ((void)0)

namespace {

struct RealVect {
    double v[3];
    explicit RealVect(double a) { v[0] = v[1] = v[2] = a; }
    RealVect(double a, double b, double c) { v[0] = a; v[1] = b; v[2] = c; }
    double &operator[](int k) { return v[k]; }
    const double &operator[](int k) const { return v[k]; }
};

// Layout-compatible with amrex::Particle<MAX_CHEM_REAL_VAR, MAX_CHEM_INT_VAR>
// as far as the loop bodies touch it.
struct RefParticle {
    double m_pos[3];
    double m_rdata[MAX_CHEM_REAL_VAR];
    int m_idata[MAX_CHEM_INT_VAR];
    RealVect pos() const { return RealVect(m_pos[0], m_pos[1], m_pos[2]); }
    double &pos(int d) { return m_pos[d]; }
    double &rdata(int k) { return m_rdata[k]; }
    int &idata(int k) { return m_idata[k]; }
    int id() const { return m_idata[intIdx::id]; }
    int cpu() const { return m_idata[intIdx::cpu]; }
};

// Neighbour iterator: dereferencing yields a particle by value with the
// periodic image shift applied to its position (a ghost copy, as AMReX's
// fillNeighbors makes them, taken when the loop starts).
struct NbrIter {
    const RefParticle *parts;
    const int32_t *idx;
    const int8_t *img;
    int64_t t;
    double lx, ly;
    bool operator!=(const NbrIter &o) const { return t != o.t; }
    NbrIter &operator++() { ++t; return *this; }
    RefParticle operator*() const
    {
        RefParticle q = parts[idx[t]];
        int sx = img[t] % 3 - 1, sy = img[t] / 3 - 1;
        if (sx) q.m_pos[0] = q.m_pos[0] + (double)sx * lx;
        if (sy) q.m_pos[1] = q.m_pos[1] + (double)sy * ly;
        return q;
    }
    int index() const { return idx[t]; }
};
// amrex::Particle<MAX_CHEM_REAL_VAR, MAX_CHEM_INT_VAR> of AMReX 22.x as the
// split loop uses it, byte for byte: pos, rdata, id, cpu, idata (448 bytes).
struct SplitParticle {
    double m_pos[3];
    double m_rdata[MAX_CHEM_REAL_VAR];
    int m_id, m_cpu;
    int m_idata[MAX_CHEM_INT_VAR];
    double &pos(int d) { return m_pos[d]; }
    double &rdata(int k) { return m_rdata[k]; }
    int &idata(int k) { return m_idata[k]; }
    int &id() { return m_id; }
    int &cpu() { return m_cpu; }
};
struct BMXParticleContainer {
    using ParticleType = SplitParticle;
};

struct NbrRange {
    NbrIter b, e;
    NbrIter begin() const { return b; }
    NbrIter end() const { return e; }
};

void to_aos(const bmxg_particles *p, std::vector<RefParticle> &a)
{
    const int64_t n = p->n;
    a.assign((size_t)n, RefParticle());
    for (int64_t i = 0; i < n; ++i) {
        RefParticle &q = a[(size_t)i];
        for (double &r : q.m_rdata) r = 0.0;
        for (int &k : q.m_idata) k = 0;
        q.m_pos[0] = p->x[i]; q.m_pos[1] = p->y[i]; q.m_pos[2] = p->z[i];
        auto R = [&](double *src, int k) { if (src) q.m_rdata[k] = src[i]; };
        auto I = [&](int32_t *src, int k) { if (src) q.m_idata[k] = src[i]; };
        R(p->radius, realIdx::radius); R(p->c_length, realIdx::c_length);
        R(p->theta, realIdx::theta); R(p->phi, realIdx::phi);
        R(p->area, realIdx::area); R(p->bond_scale, realIdx::bond_scale);
        R(p->velx, realIdx::velx); R(p->vely, realIdx::vely); R(p->velz, realIdx::velz);
        R(p->wx, realIdx::wx); R(p->wy, realIdx::wy); R(p->wz, realIdx::wz);
        I(p->cell_type, intIdx::cell_type); I(p->id, intIdx::id); I(p->cpu, intIdx::cpu);
        I(p->n_bnds, intIdx::n_bnds); I(p->position, intIdx::position);
        I(p->fuse_tip, intIdx::fuse_tip); I(p->fix_site, intIdx::fix_site);
        I(p->fuse_flag, intIdx::fuse_flag); I(p->split_flag, intIdx::split_flag);
        I(p->new_flag, intIdx::new_flag);
        const int s1[4] = {intIdx::seg1_id1, intIdx::seg2_id1, intIdx::seg3_id1, intIdx::seg4_id1};
        const int s2[4] = {intIdx::seg1_id2, intIdx::seg2_id2, intIdx::seg3_id2, intIdx::seg4_id2};
        const int st[4] = {intIdx::site1, intIdx::site2, intIdx::site3, intIdx::site4};
        for (int k = 0; k < 4; ++k) {
            if (p->seg_id1) q.m_idata[s1[k]] = p->seg_id1[k * n + i];
            if (p->seg_id2) q.m_idata[s2[k]] = p->seg_id2[k * n + i];
            if (p->site) q.m_idata[st[k]] = p->site[k * n + i];
        }
        const int dl[6] = {intIdx::dltd_site1, intIdx::dltd_site2, intIdx::dltd_id1,
                           intIdx::dltd_id2, intIdx::dltd_cpu1, intIdx::dltd_cpu2};
        for (int k = 0; k < 6; ++k)
            if (p->dltd) q.m_idata[dl[k]] = p->dltd[k * n + i];
    }
}

void from_aos(const std::vector<RefParticle> &a, bmxg_particles *p)
{
    const int64_t n = p->n;
    for (int64_t i = 0; i < n; ++i) {
        const RefParticle &q = a[(size_t)i];
        p->x[i] = q.m_pos[0]; p->y[i] = q.m_pos[1]; p->z[i] = q.m_pos[2];
        auto R = [&](double *dst, int k) { if (dst) dst[i] = q.m_rdata[k]; };
        auto I = [&](int32_t *dst, int k) { if (dst) dst[i] = q.m_idata[k]; };
        R(p->theta, realIdx::theta); R(p->phi, realIdx::phi);
        R(p->velx, realIdx::velx); R(p->vely, realIdx::vely); R(p->velz, realIdx::velz);
        R(p->wx, realIdx::wx); R(p->wy, realIdx::wy); R(p->wz, realIdx::wz);
        I(p->n_bnds, intIdx::n_bnds); I(p->position, intIdx::position);
        I(p->fix_site, intIdx::fix_site);
        I(p->fuse_flag, intIdx::fuse_flag); I(p->split_flag, intIdx::split_flag);
        I(p->new_flag, intIdx::new_flag);
        const int s1[4] = {intIdx::seg1_id1, intIdx::seg2_id1, intIdx::seg3_id1, intIdx::seg4_id1};
        const int s2[4] = {intIdx::seg1_id2, intIdx::seg2_id2, intIdx::seg3_id2, intIdx::seg4_id2};
        const int st[4] = {intIdx::site1, intIdx::site2, intIdx::site3, intIdx::site4};
        for (int k = 0; k < 4; ++k) {
            if (p->seg_id1) p->seg_id1[k * n + i] = q.m_idata[s1[k]];
            if (p->seg_id2) p->seg_id2[k * n + i] = q.m_idata[s2[k]];
            if (p->site) p->site[k * n + i] = q.m_idata[st[k]];
        }
        const int dl[6] = {intIdx::dltd_site1, intIdx::dltd_site2, intIdx::dltd_id1,
                           intIdx::dltd_id2, intIdx::dltd_cpu1, intIdx::dltd_cpu2};
        for (int k = 0; k < 6; ++k)
            if (p->dltd) p->dltd[k * n + i] = q.m_idata[dl[k]];
    }
}

std::vector<Real> force_params(const bmxg_params *prm)
{
    return {prm->bndry_width, prm->stiffness, prm->z_wall, prm->z_bndry_width,
            prm->z_stiffness, prm->z_gravity, prm->bond_strength, prm->bond_cutoff,
            prm->viscosity};
}

} // namespace

extern "C" {

// Force gather + wall force with the reference's loop body, serial over i
// (the CPU build's ParallelFor).  fc_out is 6*n planar.
int ref_forces(const bmxg_params *prm, const bmxg_geometry *geom, bmxg_particles *p,
               const int64_t *offs, const int32_t *idx, const int8_t *img,
               double *fc_out)
{
    if (!prm || !geom || !p || !offs || !fc_out) return BMXG_ERR_ARG;
    std::vector<RefParticle> parts;
    to_aos(p, parts);
    const std::vector<RefParticle> ghosts = parts; // ghost copies as of loop start
    std::vector<Real> fpar_vec = force_params(prm);
    Real *fpar = &fpar_vec[0];
    const int nrp = (int)p->n;
    const int ntot = nrp;
    std::vector<Real> fc((size_t)6 * ntot, 0.0);
    Real *fc_ptr = fc.data();
    RefParticle *pstruct = parts.data();
    const double lx = geom->prob_hi[0] - geom->prob_lo[0];
    const double ly = geom->prob_hi[1] - geom->prob_lo[1];
    struct {
        const RefParticle *g;
        const int64_t *o;
        const int32_t *ix;
        const int8_t *im;
        double lx, ly;
        NbrRange getNeighbors(int i) const
        {
            return NbrRange{NbrIter{g, ix, im, o[i], lx, ly}, NbrIter{g, ix, im, o[i + 1], lx, ly}};
        }
    } nbor_data{ghosts.data(), offs, idx, img, lx, ly};
    constexpr Real small_number = 1.0e-15;
    const int me = 0;
    const int n = 0; // substep counter passed to evaluateForce
    (void)nrp;
    for (int i = 0; i < nrp; ++i) {
        // Real neighbours are read as they are now, like the CPU build reads
        // its tile; only periodic images come from the start-of-loop copy.
        nbor_data.g = ghosts.data();
#include "force_body.inc"
    }
    (void)me; (void)n; (void)small_number;
    for (size_t k = 0; k < fc.size(); ++k) fc_out[k] = fc[k];
    from_aos(parts, p);
    return BMXG_OK;
}

// Update with the reference's loop body, then the periodic wrap of the
// trailing Redistribute (oracle port's restatement of AMReX).
void ref_update(const bmxg_geometry *geom, bmxg_particles *p, const double *fc_in, double dt)
{
    std::vector<RefParticle> parts;
    to_aos(p, parts);
    RefParticle *pstruct = parts.data();
    const int ntot = (int)p->n;
    std::vector<Real> fc(fc_in, fc_in + (size_t)6 * ntot);
    Real *fc_ptr = fc.data();
    Real subdt = dt / 1;
    for (int i = 0; i < ntot; ++i) {
#include "update_body.inc"
    }
    from_aos(parts, p);
    orc_wrap(geom, p);
}

// InitBonds with the reference's loop body (bmx_pc_interaction.cpp:577-626)
// and fixBonds, serial over i.
int ref_init_bonds(const bmxg_params *prm, const bmxg_geometry *geom, bmxg_particles *p,
                   const int64_t *offs, const int32_t *idx, const int8_t *img, double rlim_in)
{
    if (!prm || !geom || !p || !offs) return BMXG_ERR_ARG;
    std::vector<RefParticle> parts;
    to_aos(p, parts);
    const std::vector<RefParticle> ghosts = parts;
    std::vector<Real> fpar_vec = force_params(prm);
    Real *fpar = &fpar_vec[0];
    const int nrp = (int)p->n;
    RefParticle *pstruct = parts.data();
    const double lx = geom->prob_hi[0] - geom->prob_lo[0];
    const double ly = geom->prob_hi[1] - geom->prob_lo[1];
    struct {
        const RefParticle *g;
        const int64_t *o;
        const int32_t *ix;
        const int8_t *im;
        double lx, ly;
        NbrRange getNeighbors(int i) const
        {
            return NbrRange{NbrIter{g, ix, im, o[i], lx, ly}, NbrIter{g, ix, im, o[i + 1], lx, ly}};
        }
    } nbor_data{ghosts.data(), offs, idx, img, lx, ly};
    constexpr Real small_number = 1.0e-15;
    const Real rlim = rlim_in;
    for (int i = 0; i < nrp; ++i) {
#include "initbonds_body.inc"
    }
    (void)small_number;
    from_aos(parts, p);
    return BMXG_OK;
}

// ParticleExchange with the reference's loop body (bmx_pc_xchng.cpp:122-151)
// and applyIncrements, serial over i.  conc: 3 planes (A, B, C) of n, in and
// out; vol: n.  The concentrations live in the chemistry block of the real
// data (realIdx::first_data + 0..2, increments at + 3..5).
int ref_particle_exchange(const bmxg_particles *p, const int64_t *offs, const int32_t *idx, const int8_t *img,
                          const bmxg_geometry *geom, const double *vol, double *conc, double dt, const double *xp)
{
    if (!p || !offs || !vol || !conc || !xp || !geom) return BMXG_ERR_ARG;
    std::vector<RefParticle> parts;
    to_aos(p, parts);
    const int64_t n = p->n;
    for (int64_t i = 0; i < n; ++i) {
        RefParticle &q = parts[(size_t)i];
        q.m_rdata[realIdx::vol] = vol[i];
        for (int k = 0; k < 3; ++k) q.m_rdata[realIdx::first_data + k] = conc[(size_t)k * n + i];
    }
    const std::vector<RefParticle> ghosts = parts;  // neighbours as copies taken when the loop starts
    const double lx = geom->prob_hi[0] - geom->prob_lo[0];
    const double ly = geom->prob_hi[1] - geom->prob_lo[1];
    struct {
        const RefParticle *g;
        const int64_t *o;
        const int32_t *ix;
        const int8_t *im;
        double lx, ly;
        NbrRange getNeighbors(int i) const
        {
            return NbrRange{NbrIter{g, ix, im, o[i], lx, ly}, NbrIter{g, ix, im, o[i + 1], lx, ly}};
        }
    } nbor_data{ghosts.data(), offs, idx, img, lx, ly};
    std::vector<Real> xpar_vec(xp, xp + 3);
    Real *xpar = &xpar_vec[0];
    const int nrp = (int)n, ntot = nrp;
    RefParticle *pstruct = parts.data();
    const Real subdt = dt;
    // stdout of the body's diagnostics goes where the caller sends it
    for (int i = 0; i < nrp; ++i) {
#include "xchng_body.inc"
    }
    (void)ntot;
    for (int i = 0; i < nrp; ++i) {
        auto &particle = pstruct[i];
        applyIncrements(&particle.rdata(0), &particle.idata(0));
    }
    for (int64_t i = 0; i < n; ++i)
        for (int k = 0; k < 3; ++k) conc[(size_t)k * n + i] = parts[(size_t)i].m_rdata[realIdx::first_data + k];
    return BMXG_OK;
}

// Single-call entry points for unit tests.
void ref_min_distance(const double e[12], double *ti, double *tj)
{
    evaluateMinimumDistance(e[0], e[1], e[2], e[3], e[4], e[5], e[6], e[7], e[8], e[9],
                            e[10], e[11], ti, tj);
}

double ref_max_dist(const bmxg_particles *p, int64_t i, int64_t j, double bw)
{
    std::vector<RefParticle> parts;
    to_aos(p, parts);
    return maxInteractionDistance(&parts[i].rdata(0), &parts[j].rdata(0),
                                  &parts[i].idata(0), &parts[j].idata(0), bw);
}

void ref_pair_force(const bmxg_params *prm, const double r12[3], const bmxg_particles *p,
                    int64_t i, int64_t j, double v1[3], double rot1[3])
{
    std::vector<RefParticle> parts;
    to_aos(p, parts);
    std::vector<Real> fpar = force_params(prm);
    RefParticle a = parts[i], b = parts[j];
    Real d[3] = {r12[0], r12[1], r12[2]};
    Real v2[3], rot2[3];
    v1[0] = v1[1] = v1[2] = 0.0;
    rot1[0] = rot1[1] = rot1[2] = 0.0;
    evaluateForce(d, &a.rdata(0), &b.rdata(0), &a.idata(0), &b.idata(0), v1, v2, rot1, rot2,
                  fpar.data(), 0, (int)i, (int)j, 0);
}

void ref_surface_force(const bmxg_params *prm, const bmxg_particles *p, int64_t i,
                       double vel[3], double rot[3])
{
    std::vector<RefParticle> parts;
    to_aos(p, parts);
    std::vector<Real> fpar = force_params(prm);
    Real pos[3] = {p->x[i], p->y[i], p->z[i]};
    evaluateSurfaceForce(pos, &parts[i].rdata(0), &parts[i].idata(0), vel, rot, fpar.data());
}

// split_particles (src/des/bmx_split_particles.cpp:16-166) on one tile of
// BMX's own particle structs: the flag loop body (:47-54, checkSplit) and the
// fill loop body (:90-159, setNewCell / setNewSegment / setNewSegments) run as
// the serial CPU build runs them, over an engine that hands out draws[] in call
// order; the scan and the daughters' slots n + offset[i] as at :57-75.
// Daughters past cap return BMXG_ERR_CAPACITY before any write.
int ref_split_cells_aos(void *particles, int64_t n, int64_t cap, const bmxg_split_params *sp,
                        const double *draws, int64_t ndraws, int64_t next_id, int32_t my_proc,
                        int64_t *num_split, int64_t *draws_used)
{
    if (!particles || !sp || !num_split || n < 0 || cap < n) return BMXG_ERR_ARG;
    using ParticleType = SplitParticle;
    static_assert(sizeof(SplitParticle) == 448, "AMReX 22.x particle layout");
    ParticleType *pstruct = static_cast<ParticleType *>(particles);
    const int np = (int)n;
    const Real l_max_vol = sp->max_vol, l_max_len = sp->max_len, l_max_rad = sp->max_rad;
    const Real l_brnch_prob = sp->brnch_prob, l_split_prob = sp->split_prob, l_overlap = sp->overlap;
    const Real split_len = sp->split_len;
    const int l_num_reals = sp->num_reals, l_num_ints = sp->num_ints;
    long drawn = 0;
    amrex::RandomEngine engine;
    engine.u = draws;
    engine.n = (long)ndraws;
    engine.k = &drawn;
    std::vector<unsigned int> do_split((size_t)np + 1, 0u);
    unsigned int *do_split_p = do_split.data();
    for (int i = 0; i < np; ++i) {
#include "split_flag_body.inc"
    }
    std::vector<unsigned int> offsets((size_t)np + 1, 0u);
    for (int i = 0; i < np; ++i) offsets[(size_t)i + 1] = offsets[(size_t)i] + do_split[(size_t)i];
    *num_split = offsets[(size_t)np];
    if (n + *num_split > cap) return BMXG_ERR_CAPACITY;
    const long long next_pid = next_id;
    const unsigned int *poffsets = offsets.data();
    for (int pid = 0; pid < np; ++pid) {
#include "split_fill_body.inc"
    }
    if (draws_used) *draws_used = drawn;
    return BMXG_OK;
}

} // extern "C"
