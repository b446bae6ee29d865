/*
 * bmx_oracle.c -- CPU oracle of the BMX particle DEM step (plain C11).
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA product and the CPU
 * baseline of bench.py.  The product never links it.  See bmx_oracle.h for
 * what is restated from where and what is pinned against the reference's own
 * code (oracle/ref_harness.cpp).
 *
 * Build flags matter: -ffp-contract=off keeps a*b+c as two roundings (the
 * reference's release build on x86 does not contract either), so the FP64
 * results are reproducible across x86 and aarch64 hosts.
 */
#define _POSIX_C_SOURCE 199309L
#include "bmx_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_PI 3.14159265358979323846 /* M_PI as the reference uses it */

/* ------------------------------------------------------------------------ */
/* geometry (AMReX Geometry restated: dx = L/n, dxi = 1/dx)                  */
/* ------------------------------------------------------------------------ */
typedef struct {
    double plo[3], phi[3], len[3], dx[3], dxi[3];
    int n[3], per[3];
} og_t;

static int og_init(const bmxg_geometry *g, og_t *o)
{
    for (int d = 0; d < 3; ++d) {
        if (g->n_cell[d] < 1 || !(g->prob_hi[d] > g->prob_lo[d])) return BMXG_ERR_ARG;
        o->plo[d] = g->prob_lo[d];
        o->phi[d] = g->prob_hi[d];
        o->len[d] = g->prob_hi[d] - g->prob_lo[d];
        o->n[d] = g->n_cell[d];
        o->dx[d] = o->len[d] / (double)o->n[d];
        o->dxi[d] = 1.0 / o->dx[d];
        o->per[d] = g->is_periodic[d] ? 1 : 0;
        if (o->per[d] && o->n[d] < 3) return BMXG_ERR_UNSUPPORTED;
    }
    if (o->per[2]) return BMXG_ERR_UNSUPPORTED;
    return BMXG_OK;
}

/* Bin index in the coordinates of the tile box grown by one cell, as AMReX's
 * NeighborList binning computes it: (int)((x - plo)*dxi - lo) with lo = -1.
 * Clamped to [lo_c, hi_c] so that out-of-range input cannot index outside. */
static int og_bin(double x, double plo, double dxi, int lo_c, int hi_c)
{
    double v = (x - plo) * dxi - (-1.0);
    if (!(v > (double)lo_c)) return lo_c;
    if (v >= (double)hi_c + 1.0) return hi_c;
    return (int)v;
}

/* ------------------------------------------------------------------------ */
/* neighbour list (AMReX buildNeighborList + fillNeighbors restated)         */
/* ------------------------------------------------------------------------ */
typedef struct {
    int32_t src;   /* colony-local index of the source particle */
    int8_t code;   /* (sx+1) + 3*(sy+1) */
    double x, y, z;
    int bx, by, bz;
} ghost_t;

/* Builds the list of the colony occupying global indices [base, base+n). */
static int pairs_colony(const bmxg_params *prm, const og_t *g,
                        const bmxg_particles *p, int64_t base, int64_t n,
                        int64_t *offs, int32_t *idx, int8_t *img, int64_t cap,
                        int64_t *total, int nthreads)
{
    const double *X = p->x + base, *Y = p->y + base, *Z = p->z + base;
    const int NX = g->n[0] + 2, NY = g->n[1] + 2, NZ = g->n[2] + 2;
    int *bx = (int *)malloc(sizeof(int) * (size_t)(3 * n + 1));
    if (!bx) return BMXG_ERR_OOM;
    int *by = bx + n, *bz = bx + 2 * n;
    int64_t nghost = 0;
    for (int64_t i = 0; i < n; ++i) {
        bx[i] = og_bin(X[i], g->plo[0], g->dxi[0], 1, g->n[0]);
        by[i] = og_bin(Y[i], g->plo[1], g->dxi[1], 1, g->n[1]);
        bz[i] = og_bin(Z[i], g->plo[2], g->dxi[2], 1, g->n[2]);
        int mx = 1 + (g->per[0] && (bx[i] == 1 || bx[i] == g->n[0]));
        int my = 1 + (g->per[1] && (by[i] == 1 || by[i] == g->n[1]));
        nghost += mx * my - 1;
    }
    ghost_t *gh = (ghost_t *)malloc(sizeof(ghost_t) * (size_t)(nghost + 1));
    if (!gh) { free(bx); return BMXG_ERR_OOM; }
    /* ghosts in (source index, image code) order */
    int64_t ng = 0;
    for (int64_t i = 0; i < n; ++i) {
        for (int sy = -1; sy <= 1; ++sy) {
            for (int sx = -1; sx <= 1; ++sx) {
                if (sx == 0 && sy == 0) continue;
                if (sx != 0 && !(g->per[0] && bx[i] == (sx > 0 ? 1 : g->n[0]))) continue;
                if (sy != 0 && !(g->per[1] && by[i] == (sy > 0 ? 1 : g->n[1]))) continue;
                ghost_t *q = &gh[ng++];
                q->src = (int32_t)i;
                q->code = (int8_t)((sx + 1) + 3 * (sy + 1));
                q->x = sx ? X[i] + (double)sx * g->len[0] : X[i];
                q->y = sy ? Y[i] + (double)sy * g->len[1] : Y[i];
                q->z = Z[i];
                q->bx = sx ? og_bin(q->x, g->plo[0], g->dxi[0], 0, g->n[0] + 1) : bx[i];
                q->by = sy ? og_bin(q->y, g->plo[1], g->dxi[1], 0, g->n[1] + 1) : by[i];
                q->bz = bz[i];
            }
        }
    }
    /* stable counting sort of entries (reals 0..n-1, ghosts n..n+ng-1) */
    const int64_t nbins = (int64_t)NX * NY * NZ;
    int64_t *bstart = (int64_t *)calloc((size_t)(nbins + 1), sizeof(int64_t));
    int64_t *ent = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n + ng + 1));
    if (!bstart || !ent) { free(bx); free(gh); free(bstart); free(ent); return BMXG_ERR_OOM; }
#define ORC_BIN(a, b, c) (((int64_t)(a) * NY + (b)) * NZ + (c))
    for (int64_t i = 0; i < n; ++i) bstart[ORC_BIN(bx[i], by[i], bz[i]) + 1]++;
    for (int64_t k = 0; k < ng; ++k) bstart[ORC_BIN(gh[k].bx, gh[k].by, gh[k].bz) + 1]++;
    for (int64_t b = 0; b < nbins; ++b) bstart[b + 1] += bstart[b];
    {
        int64_t *fill = (int64_t *)malloc(sizeof(int64_t) * (size_t)(nbins + 1));
        if (!fill) { free(bx); free(gh); free(bstart); free(ent); return BMXG_ERR_OOM; }
        memcpy(fill, bstart, sizeof(int64_t) * (size_t)nbins);
        for (int64_t i = 0; i < n; ++i) ent[fill[ORC_BIN(bx[i], by[i], bz[i])]++] = i;
        for (int64_t k = 0; k < ng; ++k) ent[fill[ORC_BIN(gh[k].bx, gh[k].by, gh[k].bz)]++] = n + k;
        free(fill);
    }
    const double nbh = prm->neighborhood;
    /* pass 1: counts */
    int64_t *cnt = offs; /* offs[i+1] temporarily holds the count of i */
    offs[0] = 0;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 512) num_threads(nthreads)
#endif
    for (int64_t i = 0; i < n; ++i) {
        int64_t c = 0;
        for (int ii = bx[i] - 1; ii <= bx[i] + 1; ++ii)
            for (int jj = by[i] - 1; jj <= by[i] + 1; ++jj)
                for (int kk = bz[i] - 1; kk <= bz[i] + 1; ++kk) {
                    int64_t b = ORC_BIN(ii, jj, kk);
                    for (int64_t t = bstart[b]; t < bstart[b + 1]; ++t) {
                        int64_t e = ent[t];
                        if (e == i) continue;
                        double ex = e < n ? X[e] : gh[e - n].x;
                        double ey = e < n ? Y[e] : gh[e - n].y;
                        double ez = e < n ? Z[e] : gh[e - n].z;
                        double dx = X[i] - ex, dy = Y[i] - ey, dz = Z[i] - ez;
                        double r2 = dx * dx + dy * dy + dz * dz;
                        if (r2 <= nbh) ++c;
                    }
                }
        cnt[i + 1] = c;
    }
    for (int64_t i = 0; i < n; ++i) offs[i + 1] += offs[i];
    *total = offs[n];
    if (offs[n] > cap || !idx || !img) {
        free(bx); free(gh); free(bstart); free(ent);
        return (offs[n] > cap) ? BMXG_ERR_CAPACITY : BMXG_OK;
    }
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 512) num_threads(nthreads)
#endif
    for (int64_t i = 0; i < n; ++i) {
        int64_t o = offs[i];
        for (int ii = bx[i] - 1; ii <= bx[i] + 1; ++ii)
            for (int jj = by[i] - 1; jj <= by[i] + 1; ++jj)
                for (int kk = bz[i] - 1; kk <= bz[i] + 1; ++kk) {
                    int64_t b = ORC_BIN(ii, jj, kk);
                    for (int64_t t = bstart[b]; t < bstart[b + 1]; ++t) {
                        int64_t e = ent[t];
                        if (e == i) continue;
                        double ex = e < n ? X[e] : gh[e - n].x;
                        double ey = e < n ? Y[e] : gh[e - n].y;
                        double ez = e < n ? Z[e] : gh[e - n].z;
                        double dx = X[i] - ex, dy = Y[i] - ey, dz = Z[i] - ez;
                        double r2 = dx * dx + dy * dy + dz * dz;
                        if (r2 <= nbh) {
                            idx[o] = e < n ? (int32_t)e : gh[e - n].src;
                            img[o] = e < n ? (int8_t)4 : gh[e - n].code;
                            ++o;
                        }
                    }
                }
    }
#undef ORC_BIN
    free(bx); free(gh); free(bstart); free(ent);
    return BMXG_OK;
}

int orc_pairs(const bmxg_params *prm, const bmxg_geometry *geom,
              const bmxg_particles *p, int64_t *offs, int32_t *idx,
              int8_t *img, int64_t cap, int64_t *total)
{
    og_t g;
    int rc = og_init(geom, &g);
    if (rc) return rc;
    if (!prm || !p || !offs || !total || p->n < 0) return BMXG_ERR_ARG;
    return pairs_colony(prm, &g, p, 0, p->n, offs, idx, img, cap, total, 1);
}

/* ------------------------------------------------------------------------ */
/* force laws (src/chemistry/bmx_cell_interaction_K.H restated)              */
/* ------------------------------------------------------------------------ */

/* maxInteractionDistance (bmx_cell_interaction_K.H:23-40) */
static double max_dist(const bmxg_particles *p, int64_t i, int64_t j, double bw)
{
    int ti = p->cell_type[i], tj = p->cell_type[j];
    if (ti == BMXG_YEAST && tj == BMXG_YEAST) return p->radius[i] + p->radius[j] + bw;
    if (ti == BMXG_FUNGI && tj == BMXG_FUNGI) return 1.5 * (p->c_length[i] + p->c_length[j]) + bw;
    return 0.0;
}

static int in01(double t) { return t >= 0.0 && t <= 1.0; }
static double sq3(double a, double b, double c) { return a * a + b * b + c * c; }

/* closest points of two segments (bmx_cell_interaction_K.H:51-221):
 * e = {i1, i2, j1, j2} (3 each).  Same case structure, including the exact
 * zero tests on Aij and det and the unconstrained result for Aij == 0. */
void orc_min_distance(const double e[12], double *tau_i, double *tau_j)
{
    const double *a1 = e, *a2 = e + 3, *b1 = e + 6, *b2 = e + 9;
    double ri[3], rj[3], w[3];
    for (int k = 0; k < 3; ++k) {
        ri[k] = a2[k] - a1[k];
        rj[k] = b2[k] - b1[k];
        w[k] = a1[k] - b1[k];
    }
    double rirj = 0.0;
    for (int k = 0; k < 3; ++k) rirj += ri[k] * rj[k];
    const double Aii = sq3(ri[0], ri[1], ri[2]);
    const double Ajj = sq3(rj[0], rj[1], rj[2]);
    const double Aij = -rirj;
    const double det = Aii * Ajj - Aij * Aij;
    const double Bi = -(w[0] * ri[0] + w[1] * ri[1] + w[2] * ri[2]);
    const double Bj = w[0] * rj[0] + w[1] * rj[1] + w[2] * rj[2];
    double ti = 0.0, tj = 0.0;
    int search = 0;
    if (Aij == 0.0) {
        ti = Bi / Aii;
        tj = Bj / Ajj;
    } else if (det == 0.0) {
        double t0 = Bj / Ajj;
        if (in01(t0)) { ti = 0.0; tj = t0; }
        else {
            double t1 = (Bj + rirj) / Ajj;
            if (in01(t1)) { ti = 1.0; tj = t1; }
            else search = 1;
        }
    } else {
        ti = (Ajj * Bi - Aij * Bj) / det;
        tj = (Aii * Bj - Aij * Bi) / det;
        if (in01(ti)) {
            if (tj < 0.0 || tj > 1.0) {
                double t0 = Bi / Aii, t1 = (Bi + rirj) / Aii;
                if (in01(t0) && in01(t1)) {
                    double s0 = sq3(a1[0] + t0 * ri[0] - b1[0], a1[1] + t0 * ri[1] - b1[1],
                                    a1[2] + t0 * ri[2] - b1[2]);
                    double s1 = sq3(a1[0] + t1 * ri[0] - b2[0], a1[1] + t1 * ri[1] - b2[1],
                                    a1[2] + t1 * ri[2] - b2[2]);
                    if (s0 < s1) { tj = 0.0; ti = t0; } else { tj = 1.0; ti = t1; }
                } else if (in01(t0)) { tj = 0.0; ti = t0; }
                else if (in01(t1)) { tj = 1.0; ti = t1; }
                else search = 1;
            }
        } else if (in01(tj)) {
            double t0 = Bj / Ajj, t1 = (Bj + rirj) / Ajj;
            if (in01(t0) && in01(t1)) {
                double s0 = sq3(b1[0] + t0 * rj[0] - a1[0], b1[1] + t0 * rj[1] - a1[1],
                                b1[2] + t0 * rj[2] - a1[2]);
                double s1 = sq3(b1[0] + t1 * rj[0] - a2[0], b1[1] + t1 * rj[1] - a2[1],
                                b1[2] + t1 * rj[2] - a2[2]);
                if (s0 < s1) { ti = 0.0; tj = t0; } else { ti = 1.0; tj = t1; }
            } else if (in01(t0)) { ti = 0.0; tj = t0; }
            else if (in01(t1)) { ti = 1.0; tj = t1; }
            else search = 1;
        } else {
            search = 1;
        }
    }
    if (search) {
        double m[4];
        m[0] = sq3(a1[0] - b1[0], a1[1] - b1[1], a1[2] - b1[2]);
        m[1] = sq3(a1[0] - b2[0], a1[1] - b2[1], a1[2] - b2[2]);
        m[2] = sq3(a2[0] - b1[0], a2[1] - b1[1], a2[2] - b1[2]);
        m[3] = sq3(a2[0] - b2[0], a2[1] - b2[1], a2[2] - b2[2]);
        int best = 0;
        for (int k = 1; k < 4; ++k)
            if (m[k] < m[best]) best = k;
        ti = (best >= 2) ? 1.0 : 0.0;
        tj = (best & 1) ? 1.0 : 0.0;
    }
    *tau_i = ti;
    *tau_j = tj;
}

/* orientation frame R(theta, phi): columns axis, e_phi, -e_theta
 * (the rot matrices of bmx_cell_interaction_K.H:574-604). */
static void frame(double theta, double phi, double R[3][3], double nax[3])
{
    double ct = cos(theta), st = sin(theta), cp = cos(phi), sp = sin(phi);
    R[0][0] = cp * st; R[0][1] = -sp; R[0][2] = -cp * ct;
    R[1][0] = sp * st; R[1][1] = cp;  R[1][2] = -sp * ct;
    R[2][0] = ct;      R[2][1] = 0.0; R[2][2] = st;
    nax[0] = st * cp;
    nax[1] = st * sp;
    nax[2] = ct;
}

/* mobility tensors of a rod, in its own frame rotated to the lab frame:
 * a sphere of equal half-area radius a, self term 1/(6 pi a mu) and the
 * Rotne-Prager style coupling (bmx_cell_interaction_K.H:812-882). */
static void mobility(double area_full, double L, double visc, const double R[3][3],
                     double Dii[3][3], double Dij[3][3])
{
    double area = area_full / 2.0;
    double arad = sqrt(area / (4.0 * ORC_PI));
    double d0 = 1.0 / (6.0 * ORC_PI * arad * visc);
    double da, db;
    if (L > 2.0 * arad) {
        da = (L * L - 2.0 * arad * arad / 3.0) / (4.0 * ORC_PI * pow(L, 3) * visc);
        db = (L * L + 2.0 * arad * arad / 3.0) / (8.0 * ORC_PI * pow(L, 3) * visc);
    } else {
        da = (1.0 - 3.0 * L / (16.0 * arad)) / (6.0 * ORC_PI * arad * visc);
        db = (1.0 - 9.0 * L / (32.0 * arad)) / (6.0 * ORC_PI * arad * visc);
    }
    double Ds[3] = {d0, d0, d0}, Dc[3] = {da, db, db};
    /* R diag(D) R^T, accumulated as tmp = D R^T then R tmp */
    for (int which = 0; which < 2; ++which) {
        const double *dg = which ? Dc : Ds;
        double tmp[3][3], (*out)[3] = which ? Dij : Dii;
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                double s = 0.0;
                for (int k = 0; k < 3; ++k) s += (a == k ? dg[a] : 0.0) * R[b][k];
                tmp[a][b] = s;
            }
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                double s = 0.0;
                for (int k = 0; k < 3; ++k) s += R[a][k] * tmp[k][b];
                out[a][b] = s;
            }
    }
}

static int find_bond(const bmxg_particles *p, int64_t i, int32_t id, int32_t cpu)
{
    int nb = p->n_bnds[i];
    for (int k = 0; k < nb && k < 4; ++k)
        if (p->seg_id1[(int64_t)k * p->n + i] == id && p->seg_id2[(int64_t)k * p->n + i] == cpu) return k;
    return -1;
}

/* sphere-sphere cubic repulsion/adhesion (bmx_cell_interaction_K.H:243-276) */
static void sphere_pair(const bmxg_params *prm, const double r12[3], double ri,
                        double rj, double v1[3])
{
    double rS = ri + rj;
    double rA = rS + prm->bndry_width;
    double rn = sqrt(r12[0] * r12[0] + r12[1] * r12[1] + r12[2] * r12[2]);
    double ux = r12[0] / rn, uy = r12[1] / rn, uz = r12[2] / rn;
    double F = (rn < rA) ? -prm->stiffness * (rn - rA) * (rn - rA) * (rn - rS) : 0.0;
    v1[0] = F * ux;
    v1[1] = F * uy;
    v1[2] = F * uz;
}

/* rod-rod: bonded springs or closest-point contact, axial projection and the
 * mobility of segment i (bmx_cell_interaction_K.H:546-992).  Only the
 * velocity of segment i is produced: the j-side accumulation is disabled in
 * the reference (bmx_pc_interaction.cpp:251-261). */
static void rod_pair(const bmxg_params *prm, const double r12[3],
                     const bmxg_particles *p, int64_t i, int64_t j,
                     double v1[3], double rot1[3])
{
    const double rS = p->radius[i] + p->radius[j];
    const double rA = rS + prm->bndry_width;
    double kb = prm->bond_strength;
    const double scale = p->bond_scale[i] * p->bond_scale[j];
    const double Li = p->c_length[i], Lj = p->c_length[j];
    double Ri[3][3], Rj[3][3], ni[3], nj[3];
    frame(p->theta[i], p->phi[i], Ri, ni);
    frame(p->theta[j], p->phi[j], Rj, nj);
    double e[12]; /* i1, i2 (relative to j's centre), j1, j2 */
    for (int k = 0; k < 3; ++k) {
        e[k] = r12[k] - 0.5 * ni[k] * Li;
        e[3 + k] = r12[k] + 0.5 * ni[k] * Li;
        e[6 + k] = -0.5 * nj[k] * Lj;
        e[9 + k] = 0.5 * nj[k] * Lj;
    }
    double f[2][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}}; /* sites 1 and 2 of i */
    int bonded = 0;
    int ib = find_bond(p, i, p->id[j], p->cpu[j]);
    int jb = find_bond(p, j, p->id[i], p->cpu[i]);
    if (ib >= 0 && jb >= 0) {
        int si = p->site[(int64_t)ib * p->n + i];
        int sj = p->site[(int64_t)jb * p->n + j];
        int itip = p->fuse_tip ? p->fuse_tip[i] : 0;
        int jtip = p->fuse_tip ? p->fuse_tip[j] : 0;
        if ((itip > 0 && itip == si) || (jtip > 0 && jtip == sj)) kb = scale * kb;
        if ((si == 1 || si == 2) && (sj == 1 || sj == 2)) {
            const double *ea = (si == 1) ? e : e + 3;
            const double *eb = (sj == 1) ? e + 6 : e + 9;
            for (int k = 0; k < 3; ++k) f[si - 1][k] -= kb * (ea[k] - eb[k]);
            bonded = 1;
        }
    }
    if (!bonded) {
        double ti, tj;
        orc_min_distance(e, &ti, &tj);
        double d[3];
        for (int k = 0; k < 3; ++k) {
            double pi_ = e[k] + ti * (e[3 + k] - e[k]);
            double pj_ = e[6 + k] + tj * (e[9 + k] - e[6 + k]);
            d[k] = pi_ - pj_;
        }
        double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
        /* For r <= 1e-8 the reference builds a cross-product direction into
         * block-local variables that shadow the outer ones
         * (bmx_cell_interaction_K.H:744-746), so the unnormalised separation
         * is what the force uses; restated as such. */
        if (r > 1.0e-8) {
            d[0] /= r; d[1] /= r; d[2] /= r;
        }
        double F = (r < rA) ? -prm->stiffness * (r - rA) * (r - rA) * (r - rS) : 0.0;
        if (F != 0.0) {
            for (int k = 0; k < 3; ++k) {
                f[0][k] += F * d[k] * (1.0 - ti);
                f[1][k] += F * d[k] * ti;
            }
        }
    }
    /* remove the part of the site forces that moves the sites together */
    double ax[3] = {e[0] - e[3], e[1] - e[4], e[2] - e[5]};
    double ra = sqrt(ax[0] * ax[0] + ax[1] * ax[1] + ax[2] * ax[2]);
    double na[3] = {ax[0] / ra, ax[1] / ra, ax[2] / ra};
    double fn = (f[0][0] - f[1][0]) * na[0] + (f[0][1] - f[1][1]) * na[1] + (f[0][2] - f[1][2]) * na[2];
    for (int k = 0; k < 3; ++k) {
        f[0][k] -= 0.5 * fn * na[k];
        f[1][k] += 0.5 * fn * na[k];
    }
    double Dii[3][3], Dij[3][3];
    mobility(p->area[i], Li, prm->viscosity, Ri, Dii, Dij);
    double w1[3], w2[3];
    for (int a = 0; a < 3; ++a) {
        w1[a] = 0.0;
        w2[a] = 0.0;
        for (int b = 0; b < 3; ++b) {
            w1[a] += Dii[a][b] * f[0][b] + Dij[a][b] * f[1][b];
            w2[a] += Dii[a][b] * f[1][b] + Dij[a][b] * f[0][b];
        }
    }
    for (int a = 0; a < 3; ++a) v1[a] = 0.5 * (w1[a] + w2[a]);
    rot1[0] = 0.5 * (ax[1] * w1[2] - ax[2] * w1[1]);
    rot1[1] = 0.5 * (ax[2] * w1[0] - ax[0] * w1[2]);
    rot1[2] = 0.5 * (ax[0] * w1[1] - ax[1] * w1[0]);
    rot1[0] += -0.5 * (ax[1] * w2[2] - ax[2] * w2[1]);
    rot1[1] += -0.5 * (ax[2] * w2[0] - ax[0] * w2[2]);
    rot1[2] += -0.5 * (ax[0] * w2[1] - ax[1] * w2[0]);
}

void orc_pair_force(const bmxg_params *prm, const double r12[3],
                    const bmxg_particles *p, int64_t i, int64_t j,
                    double v1[3], double rot1[3])
{
    v1[0] = v1[1] = v1[2] = 0.0;
    rot1[0] = rot1[1] = rot1[2] = 0.0;
    int ti = p->cell_type[i], tj = p->cell_type[j];
    if (ti == BMXG_YEAST && tj == BMXG_YEAST)
        sphere_pair(prm, r12, p->radius[i], p->radius[j], v1);
    else if (ti == BMXG_FUNGI && tj == BMXG_FUNGI)
        rod_pair(prm, r12, p, i, j, v1, rot1);
}

/* growth-surface cubic law for one site at height z (shared by both cell
 * types, bmx_cell_interaction_K.H:1019-1030 and :1099-1121) */
static double wall_law(double z, const bmxg_params *prm, double rS)
{
    double dz = z - prm->z_wall;
    double rA = rS + prm->z_bndry_width;
    double v;
    if (dz > 0.0 && dz < rA) v = -prm->z_stiffness * (dz - rA) * (dz - rA) * (dz - rS);
    else if (dz <= 0.0) v = prm->z_stiffness * rA * rA * rS;
    else v = 0.0;
    v -= prm->z_gravity * prm->z_stiffness * rA * rA * rS;
    return v;
}

/* evaluateSurfaceForce (bmx_cell_interaction_K.H:1005-1283).  For rods the
 * mobility block of the reference (:1176-1265) is overwritten by the final
 * assignments (:1266-1281) and has no effect; it is not restated. */
void orc_surface_force(const bmxg_params *prm, const bmxg_particles *p,
                       int64_t i, double vel[3], double rot[3])
{
    vel[0] = vel[1] = vel[2] = 0.0;
    rot[0] = rot[1] = rot[2] = 0.0;
    if (p->cell_type[i] == BMXG_YEAST) {
        vel[2] = wall_law(p->z[i], prm, p->radius[i]);
    } else if (p->cell_type[i] == BMXG_FUNGI) {
        double R[3][3], na[3];
        frame(p->theta[i], p->phi[i], R, na);
        double L = p->c_length[i];
        double z1 = p->z[i] - 0.5 * na[2] * L;
        double z2 = p->z[i] + 0.5 * na[2] * L;
        double f1[3] = {0.0, 0.0, wall_law(z1, prm, p->radius[i])};
        double f2[3] = {0.0, 0.0, wall_law(z2, prm, p->radius[i])};
        double ax[3];
        for (int k = 0; k < 3; ++k) {
            double c = (k == 0) ? p->x[i] : (k == 1) ? p->y[i] : p->z[i];
            ax[k] = (c - 0.5 * na[k] * L) - (c + 0.5 * na[k] * L);
        }
        double r = sqrt(ax[0] * ax[0] + ax[1] * ax[1] + ax[2] * ax[2]);
        double u[3] = {ax[0] / r, ax[1] / r, ax[2] / r};
        double fn = (f1[0] - f2[0]) * u[0] + (f1[1] - f2[1]) * u[1] + (f1[2] - f2[2]) * u[2];
        for (int k = 0; k < 3; ++k) {
            f1[k] -= 0.5 * fn * u[k];
            f2[k] += 0.5 * fn * u[k];
        }
        for (int k = 0; k < 3; ++k) vel[k] = 0.5 * (f1[k] + f2[k]);
        for (int k = 0; k < 3; ++k) {
            f1[k] -= 0.5 * vel[k];
            f2[k] -= 0.5 * vel[k];
        }
        rot[0] = 0.5 * (ax[1] * f1[2] - ax[2] * f1[1]);
        rot[1] = 0.5 * (ax[2] * f1[0] - ax[0] * f1[2]);
        rot[2] = 0.5 * (ax[0] * f1[1] - ax[1] * f1[0]);
        rot[0] += -0.5 * (ax[1] * f2[2] - ax[2] * f2[1]);
        rot[1] += -0.5 * (ax[2] * f2[0] - ax[0] * f2[2]);
        rot[2] += -0.5 * (ax[0] * f2[1] - ax[1] * f2[0]);
    }
}

/* ------------------------------------------------------------------------ */
/* the step                                                                  */
/* ------------------------------------------------------------------------ */

static int has_rod_fields(const bmxg_particles *p)
{
    return p->c_length && p->theta && p->phi && p->area && p->bond_scale && p->id &&
           p->cpu && p->n_bnds && p->seg_id1 && p->seg_id2 && p->site;
}

/* Rod bookkeeping of the pair loop, made deterministic: each segment only
 * edits its own integers, reading its neighbours' tables as they were when
 * the step started.  Restates bmx_cell_interaction_K.H:336-545 (position
 * fix-up, dltd reset, half-bond repair of segment i; the reference's writes
 * to segment j go to a by-value copy, bmx_pc_interaction.cpp:188, and do not
 * persist). */
static int64_t rod_bookkeeping(const bmxg_params *prm, const og_t *g,
                               bmxg_particles *p, int64_t base, int64_t n,
                               const int64_t *offs, const int32_t *idx,
                               const int8_t *img, const int32_t *snap /* 13*n */)
{
    int64_t repairs = 0;
    const int64_t N = p->n;
    for (int64_t li = 0; li < n; ++li) {
        int64_t i = base + li;
        if (p->cell_type[i] != BMXG_FUNGI) continue;
        for (int64_t t = offs[li]; t < offs[li + 1]; ++t) {
            int64_t j = base + idx[t];
            if (p->cell_type[j] != BMXG_FUNGI) continue;
            int sx = img[t] % 3 - 1, sy = img[t] / 3 - 1;
            double dx = p->x[i] - (sx ? p->x[j] + (double)sx * g->len[0] : p->x[j]);
            double dy = p->y[i] - (sy ? p->y[j] + (double)sy * g->len[1] : p->y[j]);
            double dz = p->z[i] - p->z[j];
            double r2 = dx * dx + dy * dy + dz * dz;
            double rlm = max_dist(p, i, j, prm->bndry_width);
            if (!(r2 <= (rlm - 1.0e-15) * (rlm - 1.0e-15))) continue;
            /* neighbour's table at step start: snap[0]=n_bnds, 1..4 id, 5..8 cpu, 9..12 site */
            const int32_t *sj = snap + 13 * (j - base);
            const int32_t jid = p->id[j], jcpu = p->cpu[j];
            const int32_t iid = p->id[i], icpu = p->cpu[i];
            int ib;
            /* position fix-up (:338-362) */
            if (p->position && (p->position[i] == BMXG_SITE_SECOND_1 || p->position[i] == BMXG_SITE_SECOND_2)) {
                int site = (p->position[i] == BMXG_SITE_SECOND_1) ? 1 : 2;
                int nb = p->n_bnds[i];
                for (ib = 0; ib < nb; ++ib)
                    if (p->seg_id1[ib * N + i] == jid && p->seg_id2[ib * N + i] == jcpu &&
                        p->site[ib * N + i] == site) break;
                if (ib < nb && p->position[j] != BMXG_SITE_TIP) p->position[i] = BMXG_SITE_INTERIOR;
            }
            /* clean up old flags (:363-369) */
            if (p->dltd)
                for (int k = 0; k < 6; ++k) p->dltd[k * N + i] = -1;
            /* half-bond repair of i (:370-467) */
            int i_to_j = find_bond(p, i, jid, jcpu) >= 0;
            int j_to_i = 0;
            for (int k = 0; k < sj[0] && k < 4; ++k)
                if (sj[1 + k] == iid && sj[5 + k] == icpu) { j_to_i = 1; break; }
            if (!i_to_j && j_to_i) {
                int nb = p->n_bnds[i];
                int fs = p->fix_site ? p->fix_site[i] : 0;
                int isite = (fs == 0) ? (p->site[i] == 1 ? 2 : 1) : fs;
                if (nb >= 0 && nb < 4) {
                    p->seg_id1[nb * N + i] = jid;
                    p->seg_id2[nb * N + i] = jcpu;
                    p->site[nb * N + i] = isite;
                    p->n_bnds[i] = nb + 1;
                    ++repairs;
                }
            }
        }
    }
    return repairs;
}

static int forces_colony(const bmxg_params *prm, const og_t *g, bmxg_particles *p,
                         int64_t base, int64_t n, const int64_t *offs,
                         const int32_t *idx, const int8_t *img, double *fc,
                         int64_t fstride, int nthreads)
{
    const int64_t N = p->n;
    /* flag resets (bmx_pc_interaction.cpp:178-180) */
    for (int64_t li = 0; li < n; ++li) {
        int64_t i = base + li;
        if (p->fuse_flag) p->fuse_flag[i] = 0;
        if (p->split_flag) p->split_flag[i] = 0;
        if (p->new_flag) p->new_flag[i] = 0;
    }
    int any_rod = 0;
    for (int64_t li = 0; li < n && !any_rod; ++li) any_rod = (p->cell_type[base + li] == BMXG_FUNGI);
    if (any_rod) {
        if (!has_rod_fields(p)) return BMXG_ERR_ARG;
        int32_t *snap = (int32_t *)malloc(sizeof(int32_t) * (size_t)(13 * n + 1));
        if (!snap) return BMXG_ERR_OOM;
        for (int64_t li = 0; li < n; ++li) {
            int64_t i = base + li;
            int32_t *s = snap + 13 * li;
            s[0] = p->n_bnds[i];
            for (int k = 0; k < 4; ++k) {
                s[1 + k] = p->seg_id1[k * N + i];
                s[5 + k] = p->seg_id2[k * N + i];
                s[9 + k] = p->site[k * N + i];
            }
        }
        rod_bookkeeping(prm, g, p, base, n, offs, idx, img, snap);
        free(snap);
    }
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 256) num_threads(nthreads)
#endif
    for (int64_t li = 0; li < n; ++li) {
        int64_t i = base + li;
        double acc[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        for (int64_t t = offs[li]; t < offs[li + 1]; ++t) {
            int64_t j = base + idx[t];
            int sx = img[t] % 3 - 1, sy = img[t] / 3 - 1;
            double r12[3];
            r12[0] = p->x[i] - (sx ? p->x[j] + (double)sx * g->len[0] : p->x[j]);
            r12[1] = p->y[i] - (sy ? p->y[j] + (double)sy * g->len[1] : p->y[j]);
            r12[2] = p->z[i] - p->z[j];
            double r2 = r12[0] * r12[0] + r12[1] * r12[1] + r12[2] * r12[2];
            double rlm = max_dist(p, i, j, prm->bndry_width);
            if (r2 <= (rlm - 1.0e-15) * (rlm - 1.0e-15)) {
                double v1[3], w1[3];
                orc_pair_force(prm, r12, p, i, j, v1, w1);
                acc[0] += v1[0]; acc[1] += v1[1]; acc[2] += v1[2];
                acc[3] += w1[0]; acc[4] += w1[1]; acc[5] += w1[2];
            }
        }
        double vc[3], vr[3];
        orc_surface_force(prm, p, i, vc, vr);
        acc[0] += vc[0]; acc[1] += vc[1]; acc[2] += vc[2];
        acc[3] += vr[0]; acc[4] += vr[1]; acc[5] += vr[2];
        for (int c = 0; c < 6; ++c) fc[c * fstride + li] = acc[c];
    }
    /* evaluateSurfaceForce zeroes fix_site of every segment (:1060) */
    if (p->fix_site)
        for (int64_t li = 0; li < n; ++li)
            if (p->cell_type[base + li] == BMXG_FUNGI) p->fix_site[base + li] = 0;
    return BMXG_OK;
}

int orc_forces(const bmxg_params *prm, const bmxg_geometry *geom,
               bmxg_particles *p, const int64_t *offs, const int32_t *idx,
               const int8_t *img, double *fc, int nthreads)
{
    og_t g;
    int rc = og_init(geom, &g);
    if (rc) return rc;
    if (!prm || !p || !offs || !fc || p->n < 0) return BMXG_ERR_ARG;
    return forces_colony(prm, &g, p, 0, p->n, offs, idx, img, fc, p->n, nthreads < 1 ? 1 : nthreads);
}

/* AMReX enforcePeriodic restated: shift by the domain length until inside,
 * then clamp against round-off. */
static double wrap1(double x, double lo, double hi, double len)
{
    if (x > hi) {
        while (x > hi) x -= len;
        if (x < lo) x = lo;
    } else if (x < lo) {
        while (x < lo) x += len;
        if (x > hi) x = hi;
    }
    return x;
}

static void update_range(const og_t *g, bmxg_particles *p, int64_t base, int64_t n,
                         const double *fc, int64_t fstride, double dt, int nthreads)
{
    /* nsubsteps = ceil(dt/dtsolid) with dtsolid = dt -> 1 (bmx_pc_interaction.cpp:56-65) */
    const double subdt = dt / 1.0;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
    for (int64_t li = 0; li < n; ++li) {
        int64_t i = base + li;
        double v[3] = {fc[li], fc[fstride + li], fc[2 * fstride + li]};
        double w[3] = {fc[3 * fstride + li], fc[4 * fstride + li], fc[5 * fstride + li]};
        if (p->velx) p->velx[i] = v[0];
        if (p->vely) p->vely[i] = v[1];
        if (p->velz) p->velz[i] = v[2];
        if (p->wx) p->wx[i] = w[0];
        if (p->wy) p->wy[i] = w[1];
        if (p->wz) p->wz[i] = w[2];
        double x = p->x[i] + subdt * v[0];
        double y = p->y[i] + subdt * v[1];
        double z = p->z[i] + subdt * v[2];
        if (p->cell_type[i] == BMXG_FUNGI) {
            /* rotate the axis by |omega| dt about the in-plane rotation axis
             * (bmx_pc_interaction.cpp:334-431) */
            double R[3][3], na[3];
            frame(p->theta[i], p->phi[i], R, na);
            double om[3];
            for (int a = 0; a < 3; ++a) {
                om[a] = 0.0;
                for (int b = 0; b < 3; ++b) om[a] += R[b][a] * w[b];
            }
            double L = p->c_length[i];
            om[0] = 0.0;
            om[1] *= 2.0 / (L * L);
            om[2] *= 2.0 / (L * L);
            double on = sqrt(om[1] * om[1] + om[2] * om[2]);
            if (on > 0.0) {
                om[1] /= on;
                om[2] /= on;
            }
            double c = om[2], s = om[1];
            double Q[3][3] = {{1.0, 0.0, 0.0}, {0.0, c, -s}, {0.0, s, c}};
            double ang = on * subdt;
            double u[3] = {cos(ang), sin(ang), 0.0};
            double q[3];
            for (int a = 0; a < 3; ++a) {
                q[a] = 0.0;
                for (int b = 0; b < 3; ++b) q[a] += Q[b][a] * u[b];
            }
            double nd[3];
            for (int a = 0; a < 3; ++a) {
                nd[a] = 0.0;
                for (int b = 0; b < 3; ++b) nd[a] += R[a][b] * q[b];
            }
            double th = acos(nd[2]);
            double rho = sqrt(nd[0] * nd[0] + nd[1] * nd[1]);
            if (rho > 0.0) nd[0] /= rho;
            double ph = acos(nd[0]);
            if (nd[1] < 0.0) ph = 2.0 * ORC_PI - ph;
            p->theta[i] = th;
            p->phi[i] = ph;
        }
        p->x[i] = g->per[0] ? wrap1(x, g->plo[0], g->phi[0], g->len[0]) : x;
        p->y[i] = g->per[1] ? wrap1(y, g->plo[1], g->phi[1], g->len[1]) : y;
        p->z[i] = z;
    }
}

void orc_update(const bmxg_geometry *geom, bmxg_particles *p, const double *fc,
                double dt, int nthreads)
{
    og_t g;
    if (og_init(geom, &g)) return;
    update_range(&g, p, 0, p->n, fc, p->n, dt, nthreads < 1 ? 1 : nthreads);
}

void orc_wrap(const bmxg_geometry *geom, bmxg_particles *p)
{
    og_t g;
    if (og_init(geom, &g)) return;
    for (int64_t i = 0; i < p->n; ++i) {
        if (g.per[0]) p->x[i] = wrap1(p->x[i], g.plo[0], g.phi[0], g.len[0]);
        if (g.per[1]) p->y[i] = wrap1(p->y[i], g.plo[1], g.phi[1], g.len[1]);
    }
}

int orc_evolve(const bmxg_params *prm, int32_t ncol, const bmxg_geometry *geoms,
               const int64_t *offsets, bmxg_particles *p, double dt,
               int32_t nsteps, int nthreads)
{
    if (!prm || !geoms || !p || ncol < 1 || nsteps < 0 || p->n < 0) return BMXG_ERR_ARG;
    if (ncol > 1 && !offsets) return BMXG_ERR_ARG;
    if (nthreads < 1) nthreads = 1;
    int rc = BMXG_OK;
    for (int32_t c = 0; c < ncol && rc == BMXG_OK; ++c) {
        og_t g;
        rc = og_init(&geoms[c], &g);
        if (rc) return rc;
        int64_t base = offsets ? offsets[c] : 0;
        int64_t n = offsets ? offsets[c + 1] - offsets[c] : p->n;
        if (n <= 0) continue;
        int64_t *offs = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n + 1));
        double *fc = (double *)malloc(sizeof(double) * (size_t)(6 * n));
        int64_t cap = 64 * n + 64;
        int32_t *idx = (int32_t *)malloc(sizeof(int32_t) * (size_t)cap);
        int8_t *img = (int8_t *)malloc((size_t)cap);
        if (!offs || !fc || !idx || !img) { free(offs); free(fc); free(idx); free(img); return BMXG_ERR_OOM; }
        for (int32_t s = 0; s < nsteps && rc == BMXG_OK; ++s) {
            int64_t total = 0;
            rc = pairs_colony(prm, &g, p, base, n, offs, idx, img, cap, &total, nthreads);
            if (rc == BMXG_ERR_CAPACITY) {
                free(idx); free(img);
                cap = total + total / 4 + 64;
                idx = (int32_t *)malloc(sizeof(int32_t) * (size_t)cap);
                img = (int8_t *)malloc((size_t)cap);
                if (!idx || !img) { rc = BMXG_ERR_OOM; break; }
                rc = pairs_colony(prm, &g, p, base, n, offs, idx, img, cap, &total, nthreads);
            }
            if (rc) break;
            rc = forces_colony(prm, &g, p, base, n, offs, idx, img, fc, n, nthreads);
            if (rc) break;
            update_range(&g, p, base, n, fc, n, dt, nthreads);
        }
        free(offs); free(fc); free(idx); free(img);
    }
    return rc;
}

double orc_time_evolve(const bmxg_params *prm, int32_t ncol,
                       const bmxg_geometry *geoms, const int64_t *offsets,
                       bmxg_particles *p, double dt, int32_t nsteps, int nthreads)
{
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    int rc = orc_evolve(prm, ncol, geoms, offsets, p, dt, nsteps, nthreads);
    clock_gettime(CLOCK_MONOTONIC, &t1);
    if (rc) return -1.0;
    return (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
}

/* ------------------------------------------------------------------------ */
/* InitBonds (src/des/bmx_pc_interaction.cpp:500-668) with fixBonds          */
/* (src/chemistry/bmx_cell_interaction_K.H:1285-1444), restated              */
/* ------------------------------------------------------------------------ */

/* For every FUNGI segment i, in list order over its gated FUNGI neighbours
 * j, the first pair of ends (i1-j1, i2-j1, i1-j2, i2-j2) closer than rlim
 * appends (id_j, cpu_j, site of i) to i's bond table.  fixBonds also writes
 * j's table, but j is the loop's by-value copy (bmx_pc_interaction.cpp:591),
 * so only i's table changes.  fixBonds does not check the table's capacity
 * (it would write past seg4); here a fifth bond is not stored and counted
 * in *overflow instead. */
int orc_init_bonds(const bmxg_params *prm, const bmxg_geometry *geom, bmxg_particles *p,
                   const int64_t *offs, const int32_t *idx, const int8_t *img, double rlim,
                   int64_t *added, int64_t *overflow)
{
    og_t g;
    int rc = og_init(geom, &g);
    if (rc) return rc;
    if (!prm || !p || !offs || p->n < 0) return BMXG_ERR_ARG;
    if (!has_rod_fields(p)) return BMXG_ERR_ARG;
    const int64_t N = p->n;
    int64_t nadd = 0, nover = 0;
    for (int64_t i = 0; i < N; ++i) {
        if (p->cell_type[i] != BMXG_FUNGI) continue;
        for (int64_t t = offs[i]; t < offs[i + 1]; ++t) {
            int64_t j = idx[t];
            if (p->cell_type[j] != BMXG_FUNGI) continue;
            int sx = img[t] % 3 - 1, sy = img[t] / 3 - 1;
            double r12[3];
            r12[0] = p->x[i] - (sx ? p->x[j] + (double)sx * g.len[0] : p->x[j]);
            r12[1] = p->y[i] - (sy ? p->y[j] + (double)sy * g.len[1] : p->y[j]);
            r12[2] = p->z[i] - p->z[j];
            double r2 = r12[0] * r12[0] + r12[1] * r12[1] + r12[2] * r12[2];
            double rlm = max_dist(p, i, j, prm->bndry_width);
            if (!(r2 <= (rlm - 1.0e-15) * (rlm - 1.0e-15))) continue;
            double Ri[3][3], Rj[3][3], ni[3], nj[3];
            frame(p->theta[i], p->phi[i], Ri, ni);
            frame(p->theta[j], p->phi[j], Rj, nj);
            double e[4][3];  /* i1, i2, j1, j2 (j at the origin) */
            for (int k = 0; k < 3; ++k) {
                e[0][k] = r12[k] - 0.5 * ni[k] * p->c_length[i];
                e[1][k] = r12[k] + 0.5 * ni[k] * p->c_length[i];
                e[2][k] = -0.5 * nj[k] * p->c_length[j];
                e[3][k] = 0.5 * nj[k] * p->c_length[j];
            }
            /* (site of i, site of j) in the order fixBonds tries them */
            static const int order[4][2] = {{1, 1}, {2, 1}, {1, 2}, {2, 2}};
            for (int m = 0; m < 4; ++m) {
                const double *a = e[order[m][0] - 1], *b = e[1 + order[m][1]];
                double dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
                double r = sqrt(dx * dx + dy * dy + dz * dz);
                if (r < rlim) {
                    int nb = p->n_bnds[i];
                    if (nb >= 0 && nb < 4) {
                        p->seg_id1[nb * N + i] = p->id[j];
                        p->seg_id2[nb * N + i] = p->cpu[j];
                        p->site[nb * N + i] = order[m][0];
                        p->n_bnds[i] = nb + 1;
                        ++nadd;
                    } else {
                        ++nover;
                    }
                    break;
                }
            }
        }
    }
    if (added) *added = nadd;
    if (overflow) *overflow = nover;
    return BMXG_OK;
}

/* ParticleExchange (bmx_pc_xchng.cpp:13-257; initExchange, evaluateExchange,
 * applyIncrements of bmx_chem_K.H:1949-2126), one substep over the given
 * neighbour list.  conc: 3 planes (A, B, C) of n, updated in place; vol: n.
 * For each FUNGI segment i: its increments start at zero; every listed
 * FUNGI neighbour j that i and j both list as bonded moves
 * d = (c_i - c_j) * area * mt * dt, area the mean septum cross-section
 * pi (r_i^2 + r_j^2) / 2, clamped so that neither side can go negative in
 * one bond's share (c / n_bnds), and i's increment changes by -d / vol_i
 * (the write to j's increment lands on the by-value neighbour copy and is
 * lost, as in the reference).  Then every segment adds its increments. */
int orc_particle_exchange(const bmxg_geometry *geom, const bmxg_particles *p, const int64_t *offs,
                          const int32_t *idx, const double *vol, double *conc, double dt,
                          const double xpar[3])
{
    (void)geom;
    if (!p || !offs || !vol || !conc || !xpar || p->n < 0) return BMXG_ERR_ARG;
    if (!has_rod_fields(p)) return BMXG_ERR_ARG;
    const int64_t N = p->n;
    double *inc = (double *)calloc((size_t)(3 * N + 1), sizeof(double));
    if (!inc) return BMXG_ERR_OOM;
    const double pi = 3.14159265358979323846;
    for (int64_t i = 0; i < N; ++i) {
        if (p->cell_type[i] != BMXG_FUNGI) continue;
        double *ci = inc + 3 * i;  /* initExchange */
        ci[0] = ci[1] = ci[2] = 0.0;
        for (int64_t t = offs[i]; t < offs[i + 1]; ++t) {
            const int64_t j = idx[t];
            if (p->cell_type[j] != BMXG_FUNGI) continue;
            const int ib = find_bond(p, i, p->id[j], p->cpu[j]);
            const int jb = find_bond(p, j, p->id[i], p->cpu[i]);
            if (ib < 0 || jb < 0) continue;
            const double a1 = conc[i], b1 = conc[N + i], c1 = conc[2 * N + i];
            const double a2 = conc[j], b2 = conc[N + j], c2 = conc[2 * N + j];
            const double r1 = p->radius[i], r2 = p->radius[j];
            const double area1 = pi * r1 * r1, area2 = pi * r2 * r2;
            const double v1 = vol[i], v2 = vol[j];
            const double area = 0.5 * (area1 + area2);
            double dA = (a1 - a2) * area * xpar[0] * dt;
            double dB = (b1 - b2) * area * xpar[1] * dt;
            double dC = (c1 - c2) * area * xpar[2] * dt;
            const double ni = (double)p->n_bnds[i], nj = (double)p->n_bnds[j];
            if (dA / v1 > a1 / ni) dA = a1 * v1 / ni;
            if (-dA / v2 > a2 / nj) dA = -a2 * v2 / nj;
            if (dB / v1 > b1 / ni) dB = b1 * v1 / ni;
            if (-dB / v2 > b2 / nj) dB = -b2 * v2 / nj;
            if (dC / v1 > c1 / ni) dC = c1 * v1 / ni;
            if (-dC / v2 > c2 / nj) dC = -c2 * v2 / nj;
            ci[0] -= dA / v1;
            ci[1] -= dB / v1;
            ci[2] -= dC / v1;
        }
    }
    for (int64_t i = 0; i < N; ++i) {  /* applyIncrements */
        if (p->cell_type[i] != BMXG_FUNGI) continue;
        conc[i] += inc[3 * i];
        conc[N + i] += inc[3 * i + 1];
        conc[2 * N + i] += inc[3 * i + 2];
    }
    free(inc);
    return BMXG_OK;
}

/* ------------------------------------------------------------------------ */
/* cell division (split_particles)                                           */
/* ------------------------------------------------------------------------ */

/* realIdx / intIdx positions the division touches (bmx_chem.H:38-118) */
enum { SR_radius = 0, SR_c_length = 1, SR_theta = 2, SR_phi = 3, SR_area = 4, SR_vol = 5, SR_dadt = 21,
       SR_dvdt = 22, SR_bond_scale = 24, SR_first = 25 };
enum { SI_cell_type = 5, SI_n_bnds = 6, SI_seg1_id1 = 7, SI_seg2_id1 = 8, SI_seg3_id1 = 9, SI_seg4_id1 = 10,
       SI_seg1_id2 = 11, SI_seg2_id2 = 12, SI_seg3_id2 = 13, SI_seg4_id2 = 14, SI_site1 = 15, SI_site2 = 16,
       SI_site3 = 17, SI_site4 = 18, SI_position = 19, SI_fuse_flag = 20, SI_split_flag = 21,
       SI_new_flag = 22, SI_fuse_id = 23, SI_fuse_cpu = 24, SI_fuse_tip = 25, SI_dltd_site1 = 26,
       SI_fix_site = 32, SI_id = 33, SI_cpu = 34, SI_first = 35 };

/* SplitMix64 (Steele, Lea and Flood, OOPSLA 2014) on the counter (cpu, id, j),
 * 53 bits to a double in [0, 1): the draws of the library's seeded mode. */
double orc_split_uniform(uint64_t seed, int32_t id, int32_t cpu, int32_t j)
{
    const uint64_t key = ((uint64_t)(uint32_t)cpu << 32) | (uint64_t)(uint32_t)id;
    uint64_t z = seed + UINT64_C(0x9E3779B97F4A7C15) * (key * 2u + (uint64_t)j + 1u);
    z = (z ^ (z >> 30)) * UINT64_C(0xBF58476D1CE4E5B9);
    z = (z ^ (z >> 27)) * UINT64_C(0x94D049BB133111EB);
    z ^= z >> 31;
    return (double)(z >> 11) * 0x1.0p-53;
}

/* one record's views */
typedef struct {
    double *p, *r;
    int *id, *q;
} orec_t;

/* the draws of one cell: the caller's sequence from *next, or the counter
 * generator at (id, cpu, j0 + k) */
typedef struct {
    const double *seq;
    int64_t *next;
    uint64_t seed;
    int id, cpu, j;
} odraw_t;

static double odraw(odraw_t *d)
{
    if (d->seq) return d->seq[(*d->next)++];
    return orc_split_uniform(d->seed, d->id, d->cpu, d->j++);
}

/* checkSplit (bmx_chem_K.H:23-69): the draw it takes (FUNGI tip at the radius
 * limit, segment behind a tip) and the new-particle count it returns */
static int ocheck_draws(const bmxg_split_params *sp, const orec_t *m)
{
    if (m->q[SI_cell_type] != BMXG_FUNGI) return 0;
    if (m->q[SI_position] == BMXG_SITE_TIP) return m->r[SR_radius] >= sp->max_rad;
    return m->q[SI_position] == BMXG_SITE_SECOND_1 || m->q[SI_position] == BMXG_SITE_SECOND_2;
}

static int odecide(const bmxg_split_params *sp, const orec_t *m, double x)
{
    const int ct = m->q[SI_cell_type];
    if (ct == BMXG_YEAST) return m->r[SR_vol] > sp->max_vol ? 1 : 0;
    if (ct != BMXG_FUNGI) return 0;
    if (m->q[SI_position] == BMXG_SITE_TIP) {
        if (!(m->r[SR_radius] >= sp->max_rad) || !(m->r[SR_c_length] >= sp->max_len)) return 0;
        return (x > sp->split_prob || m->q[SI_n_bnds] == 0) ? 1 : 2;
    }
    if (m->q[SI_position] == BMXG_SITE_SECOND_1 || m->q[SI_position] == BMXG_SITE_SECOND_2)
        return x < sp->brnch_prob ? 1 : 0;
    return 0;
}

/* setNewCell (bmx_chem_K.H:383-440): mother and daughter apart by
 * (1 - overlap) r / 2 each along n = (sin t cos p, sin t sin p, cos t),
 * cos t = 2 u1 - 1, p = 2 pi u2; half the volume each, radius, area and dadt
 * of that volume, the daughter's bond_scale and fuse_tip reset, both cells'
 * species increments first_data + 6..8 halved */
static void odivide_cell(const bmxg_split_params *sp, orec_t *m, orec_t *d, odraw_t *u)
{
    const double x = m->p[0], y = m->p[1], z = m->p[2];
    double radius = d->r[SR_radius];
    const double theta = acos(2.0 * odraw(u) - 1.0);
    const double phi = 2.0 * ORC_PI * odraw(u);
    const double nx = sin(theta) * cos(phi), ny = sin(theta) * sin(phi), nz = cos(theta);
    const double half = (1.0 - sp->overlap) * 0.5;
    d->p[0] = x + half * nx * radius;
    d->p[1] = y + half * ny * radius;
    d->p[2] = z + half * nz * radius;
    m->p[0] = x - half * nx * radius;
    m->p[1] = y - half * ny * radius;
    m->p[2] = z - half * nz * radius;
    const double volume = m->r[SR_vol] / 2.0;
    radius = pow(3.0 * volume / (4.0 * ORC_PI), 1.0 / 3.0);
    const double area = 4.0 * ORC_PI * radius * radius;
    const double dadt = 2.0 * m->r[SR_dvdt] / radius;
    m->r[SR_vol] = d->r[SR_vol] = volume;
    m->r[SR_area] = d->r[SR_area] = area;
    m->r[SR_dadt] = d->r[SR_dadt] = dadt;
    m->r[SR_radius] = d->r[SR_radius] = radius;
    d->r[SR_bond_scale] = 1.0;
    d->q[SI_fuse_tip] = 0;
    for (int j = 6; j < 9; ++j) {
        m->r[SR_first + j] = 0.5 * m->r[SR_first + j];
        d->r[SR_first + j] = 0.5 * d->r[SR_first + j];
    }
}

/* polar angles as the reference recovers a direction's: t = acos(z),
 * p = acos(x / sin t), 2 pi - p for y < 0, p = 0 on the axis */
static void oangles(double x, double y, double z, double *t, double *st, double *p)
{
    *t = acos(z);
    *st = sin(*t);
    *p = 0.0;
    if (*st != 0.0) {
        *p = acos(x / *st);
        if (y < 0.0) *p = 2.0 * ORC_PI - *p;
    }
}

/* a direction within 0.1 rad of the x axis (t = 0.1 u1, p = 2 pi u2) turned
 * by the rotation that takes the x axis to (sin gt cos gp, sin gt sin gp,
 * cos gt) */
static void oaround(double gst, double gct, double gphi, odraw_t *u, double g[3])
{
    const double gcp = cos(gphi), gsp = sin(gphi);
    const double R[3][3] = {{gcp * gst, -gsp, -gcp * gct}, {gsp * gst, gcp, -gsp * gct}, {gct, 0.0, gst}};
    const double rt = 0.1 * odraw(u);
    const double rp = 2.0 * ORC_PI * odraw(u);
    const double v[3] = {cos(rt), sin(rt) * sin(rp), sin(rt) * cos(rp)};
    for (int k = 0; k < 3; ++k) g[k] = R[k][0] * v[0] + R[k][1] * v[1] + R[k][2] * v[2];
}

static void otip_flags(int *q, int dltd, int newf)
{
    q[SI_position] = BMXG_SITE_TIP;
    q[SI_fuse_flag] = 0;
    q[SI_split_flag] = 0;
    if (newf) q[SI_new_flag] = 0;
    q[SI_fuse_id] = -1;
    q[SI_fuse_cpu] = -1;
    if (dltd)
        for (int j = 0; j < 6; ++j) q[SI_dltd_site1 + j] = -1;
}

static void ocylinder(double *r)
{
    const double L = r[SR_c_length], a = r[SR_radius];
    r[SR_vol] = ORC_PI * a * a * L;
    r[SR_area] = 2.0 * ORC_PI * a * L + 2.0 * ORC_PI * a * a;
}

static void odir(const double *r, double n[3])
{
    n[0] = sin(r[SR_theta]) * cos(r[SR_phi]);
    n[1] = sin(r[SR_theta]) * sin(r[SR_phi]);
    n[2] = cos(r[SR_theta]);
}

/* setNewSegment (bmx_chem_K.H:457-1011).  The gradient is forced to zero
 * (:468-473), so a tip grows along itself and a side branch leaves at +-45
 * degrees (draw > 0.5: +) in the xy plane before the 0.1 rad scatter.
 *  isolated (no bonds): two halves a quarter length either side, bonded;
 *  tip: keeps split_len at its bonded end; the new tip of the remaining
 *       length starts at the mother's new free end;
 *  behind a tip: a 5e-4 branch at the end the tip hangs on; both radii shrink
 *       to sqrt(V / (pi 2 L)) (the daughter still holds the mother's length,
 *       :939).
 * Bond tables, sites, positions and the flags of a new tip as the reference
 * sets them; volume and area of both from length and radius. */
static void odivide_segment(const bmxg_split_params *sp, orec_t *m, orec_t *d, odraw_t *u, int id, int cpu)
{
    const int nbnd = m->q[SI_n_bnds], position = m->q[SI_position];
    double n[3];
    odir(m->r, n);
    const double c = m->r[SR_c_length];
    double x[3] = {m->p[0], m->p[1], m->p[2]};
    if (nbnd == 0) {
        for (int k = 0; k < 3; ++k) {
            m->p[k] = x[k] + 0.25 * c * n[k];
            d->p[k] = x[k] - 0.25 * c * n[k];
        }
        m->r[SR_c_length] = d->r[SR_c_length] = 0.5 * c;
        m->q[SI_n_bnds] = 1;
        m->q[SI_seg1_id1] = id;
        m->q[SI_seg1_id2] = cpu;
        m->q[SI_site1] = 1;
        otip_flags(m->q, 1, 1);
        d->q[SI_n_bnds] = 1;
        d->q[SI_seg1_id1] = m->q[SI_id];
        d->q[SI_seg1_id2] = m->q[SI_cpu];
        d->q[SI_site1] = 2;
        otip_flags(d->q, 1, 1);
        d->q[SI_fix_site] = 0;
        for (int j = 6; j < 9; ++j) {
            m->r[SR_first + j] = 0.5 * m->r[SR_first + j];
            d->r[SR_first + j] = 0.5 * d->r[SR_first + j];
        }
    } else if (position == BMXG_SITE_TIP) {
        const int bsite = m->q[SI_site1];
        double gt, gst, gp, g[3], nt, nst, np;
        oangles(n[0], n[1], n[2], &gt, &gst, &gp);
        oaround(gst, n[2], gp, u, g);
        const double sl = sp->split_len, rest = c - sl;
        double e[3], f[3];
        if (bsite == 1) {  /* keep the site-1 end, grow from the new site 2 */
            for (int k = 0; k < 3; ++k) {
                const double a = x[k] - 0.5 * c * n[k];
                e[k] = a + sl * n[k];
                m->p[k] = 0.5 * (a + e[k]);
                f[k] = e[k] + g[k] * rest;
            }
            m->q[nbnd == 1 ? SI_site2 : SI_site3] = 2;
            m->q[SI_position] = BMXG_SITE_SECOND_2;
        } else {
            for (int k = 0; k < 3; ++k) {
                const double b = x[k] + 0.5 * c * n[k];
                e[k] = b - sl * n[k];
                m->p[k] = 0.5 * (e[k] + b);
                f[k] = e[k] - g[k] * rest;
            }
            m->q[nbnd == 1 ? SI_site2 : SI_site3] = 1;
            m->q[SI_position] = BMXG_SITE_SECOND_1;
        }
        m->r[SR_c_length] = sl;
        for (int k = 0; k < 3; ++k) d->p[k] = 0.5 * (e[k] + f[k]);
        d->r[SR_c_length] = rest;
        oangles(g[0], g[1], g[2], &nt, &nst, &np);
        d->r[SR_theta] = nt;
        d->r[SR_phi] = np;
        d->q[SI_site1] = bsite == 1 ? 1 : 2;
        otip_flags(d->q, bsite == 1, 1);
        d->q[SI_fix_site] = 0;
        m->q[SI_n_bnds] = nbnd == 1 ? 2 : 3;
        m->q[nbnd == 1 ? SI_seg2_id1 : SI_seg3_id1] = id;
        m->q[nbnd == 1 ? SI_seg2_id2 : SI_seg3_id2] = cpu;
        d->q[SI_n_bnds] = 1;
        d->q[SI_seg1_id1] = m->q[SI_id];
        d->q[SI_seg1_id2] = m->q[SI_cpu];
        for (int j = 6; j < 9; ++j) d->r[SR_first + j] = 0.0;
    } else if (position == BMXG_SITE_SECOND_1 || position == BMXG_SITE_SECOND_2) {
        const double phi = m->r[SR_phi];
        const double tphi = phi + (odraw(u) > 0.5 ? 0.25 * ORC_PI : -0.25 * ORC_PI);
        double gt, gst, gp, g[3], nt, nst, np;
        oangles(cos(tphi), sin(tphi), 0.0, &gt, &gst, &gp);
        oaround(gst, 0.0, gp, u, g);
        oangles(g[0], g[1], g[2], &nt, &nst, &np);
        const double bl = 0.0005;
        const int s1 = position == BMXG_SITE_SECOND_1;
        if (nbnd == 2) m->q[SI_site3] = s1 ? 1 : 2;
        else if (nbnd == 3) m->q[SI_site4] = s1 ? 1 : 2;
        for (int k = 0; k < 3; ++k) {
            const double end = s1 ? x[k] - 0.5 * c * n[k] : x[k] + 0.5 * c * n[k];
            const double far = s1 ? end - g[k] * bl : end + g[k] * bl;
            d->p[k] = 0.5 * (end + far);
        }
        d->q[SI_site1] = d->q[SI_site2] = s1 ? 2 : 1;
        const double a0 = m->r[SR_radius];
        const double v0 = c * a0 * a0 * ORC_PI;
        d->r[SR_theta] = nt;
        d->r[SR_phi] = np;
        const double a1 = sqrt(v0 / (ORC_PI * (c + d->r[SR_c_length])));
        m->r[SR_radius] = d->r[SR_radius] = a1;
        d->r[SR_c_length] = bl;
        m->q[SI_n_bnds] = nbnd == 2 ? 3 : 4;
        m->q[nbnd == 2 ? SI_seg3_id1 : SI_seg4_id1] = id;
        m->q[nbnd == 2 ? SI_seg3_id2 : SI_seg4_id2] = cpu;
        d->q[SI_n_bnds] = 2;
        d->q[SI_seg1_id1] = m->q[SI_id];
        d->q[SI_seg1_id2] = m->q[SI_cpu];
        d->q[SI_seg2_id1] = m->q[nbnd == 2 ? SI_seg2_id1 : SI_seg3_id1];
        d->q[SI_seg2_id2] = m->q[nbnd == 2 ? SI_seg2_id2 : SI_seg3_id2];
        otip_flags(d->q, 1, 1);
        d->q[SI_fix_site] = 0;
        m->q[SI_position] = BMXG_SITE_INTERIOR;
        for (int j = 6; j < 9; ++j) d->r[SR_first + j] = 0.0;
    }
    d->q[SI_id] = id;
    d->q[SI_cpu] = cpu;
    ocylinder(m->r);
    ocylinder(d->r);
    d->r[SR_bond_scale] = 1.0;
    d->q[SI_fuse_tip] = 0;
}

/* setNewSegments (bmx_chem_K.H:2129-2494): a tip keeps split_len at its bonded
 * end; two tips of half the rest each leave its free end at phi +- 45 degrees
 * in the xy plane (then the 0.1 rad scatter), bonded to the mother and to each
 * other */
static void odivide_tip_in_two(const bmxg_split_params *sp, orec_t *m, orec_t *d1, orec_t *d2, odraw_t *u,
                               int id1, int cpu1, int id2, int cpu2)
{
    double n[3];
    odir(m->r, n);
    const double phi = m->r[SR_phi];
    double gt, gst1, gp1, gst2, gp2, g1[3], g2[3], t1, st1, p1, t2, st2, p2;
    oangles(cos(phi + 0.25 * ORC_PI), sin(phi + 0.25 * ORC_PI), 0.0, &gt, &gst1, &gp1);
    oangles(cos(phi - 0.25 * ORC_PI), sin(phi - 0.25 * ORC_PI), 0.0, &gt, &gst2, &gp2);
    oaround(gst1, 0.0, gp1, u, g1);
    oaround(gst2, 0.0, gp2, u, g2);
    oangles(g1[0], g1[1], g1[2], &t1, &st1, &p1);
    oangles(g2[0], g2[1], g2[2], &t2, &st2, &p2);
    const double c = m->r[SR_c_length];
    const double half = 0.5 * (c - sp->split_len), keep = c - 2.0 * half;
    const int s1 = m->q[SI_site1] == 1;
    for (int k = 0; k < 3; ++k) {
        const double x = m->p[k];
        const double a = s1 ? x - 0.5 * c * n[k] : x + 0.5 * c * n[k];  /* the kept end */
        const double b = s1 ? a + keep * n[k] : a - keep * n[k];        /* the new free end */
        m->p[k] = 0.5 * (a + b);
        d1->p[k] = 0.5 * (b + (s1 ? b + g1[k] * half : b - g1[k] * half));
        d2->p[k] = 0.5 * (b + (s1 ? b + g2[k] * half : b - g2[k] * half));
    }
    const int site = s1 ? 1 : 2, msite = s1 ? 2 : 1;
    int *q1 = d1->q, *q2 = d2->q;
    q1[SI_site1] = q1[SI_site2] = site;
    q1[SI_seg1_id1] = m->q[SI_id];
    q1[SI_seg1_id2] = m->q[SI_cpu];
    q1[SI_seg2_id1] = id2;
    q1[SI_seg2_id2] = cpu2;
    q1[SI_n_bnds] = 2;
    q2[SI_site1] = q2[SI_site2] = site;
    q2[SI_seg1_id1] = m->q[SI_id];
    q2[SI_seg1_id2] = m->q[SI_cpu];
    q2[SI_seg2_id1] = id1;
    q2[SI_seg2_id2] = cpu1;
    q2[SI_n_bnds] = 2;
    const int one = m->q[SI_n_bnds] == 1;
    m->q[one ? SI_site2 : SI_site3] = msite;
    m->q[one ? SI_seg2_id1 : SI_seg3_id1] = id1;
    m->q[one ? SI_seg2_id2 : SI_seg3_id2] = cpu1;
    m->q[one ? SI_site3 : SI_site4] = msite;
    m->q[one ? SI_seg3_id1 : SI_seg4_id1] = id2;
    m->q[one ? SI_seg3_id2 : SI_seg4_id2] = cpu2;
    m->q[SI_n_bnds] = one ? 3 : 4;
    m->r[SR_c_length] = keep;
    d1->r[SR_c_length] = d2->r[SR_c_length] = half;
    d1->r[SR_theta] = t1;
    d1->r[SR_phi] = p1;
    d2->r[SR_theta] = t2;
    d2->r[SR_phi] = p2;
    otip_flags(q1, 1, 0);
    q1[SI_fix_site] = 0;
    otip_flags(q2, 1, 0);
    q2[SI_fix_site] = 0;
    m->q[SI_position] = BMXG_SITE_INTERIOR;
    q1[SI_id] = id1;
    q1[SI_cpu] = cpu1;
    q2[SI_id] = id2;
    q2[SI_cpu] = cpu2;
    ocylinder(m->r);
    ocylinder(d1->r);
    d1->r[SR_bond_scale] = 1.0;
    q1[SI_fuse_tip] = 0;
    ocylinder(d2->r);
    d2->r[SR_bond_scale] = 1.0;
    q2[SI_fuse_tip] = 0;
}

/* split_particles (bmx_split_particles.cpp:16-166) run serially: checkSplit
 * for every particle in array order (taking its draw there), the exclusive
 * scan of the new-particle counts, and the fill loop in array order, new
 * particle k at record n + k with id next_id + k, the divisions taking their
 * draws in that order. */
int orc_split_cells_aos(const bmxg_split_params *sp, void *particles, int64_t n, int64_t cap,
                        int32_t nreal, int32_t nint, const double *draws, int64_t ndraws,
                        uint64_t seed, int64_t next_id, int32_t my_proc, int64_t *num_split)
{
    if (!sp || !num_split || n < 0 || cap < n) return BMXG_ERR_ARG;
    *num_split = 0;
    if (nreal < SR_first + 9 || nint < SI_first) return BMXG_ERR_ARG;
    if (sp->num_reals < 0 || sp->num_ints < 0 || SR_first + sp->num_reals > nreal ||
        SI_first + sp->num_ints > nint)
        return BMXG_ERR_ARG;
    if (n == 0) return BMXG_OK;
    if (!particles) return BMXG_ERR_ARG;
    const size_t off_r = 3 * sizeof(double);
    const size_t off_id = off_r + (size_t)nreal * sizeof(double);
    const size_t off_i = off_id + 2 * sizeof(int);
    const size_t stride = (off_i + (size_t)nint * sizeof(int) + 7) / 8 * 8;
    unsigned char *base = (unsigned char *)particles;
#define OREC(i) ((orec_t){(double *)(base + (size_t)(i) * stride), (double *)(base + (size_t)(i) * stride + off_r), \
                          (int *)(base + (size_t)(i) * stride + off_id), (int *)(base + (size_t)(i) * stride + off_i)})
    signed char *nnew = (signed char *)malloc((size_t)n);
    if (!nnew) return BMXG_ERR_OOM;
    int64_t next = 0, total = 0, need = 0;
    for (int64_t i = 0; i < n; ++i) {
        const orec_t m = OREC(i);
        double x = 0.0;
        if (ocheck_draws(sp, &m)) {
            if (draws && next >= ndraws) {
                free(nnew);
                return BMXG_ERR_ARG;
            }
            x = draws ? draws[next++] : orc_split_uniform(seed, m.id[0], m.id[1], 0);
        }
        nnew[i] = (signed char)odecide(sp, &m, x);
        total += nnew[i];
        if (nnew[i] == 2) need += 4;
        else if (nnew[i] == 1)
            need += m.q[SI_cell_type] == BMXG_YEAST ? 2
                  : (m.q[SI_n_bnds] == 0 ? 0 : (m.q[SI_position] == BMXG_SITE_TIP ? 2 : 3));
    }
    *num_split = total;
    if (total == 0 || n + total > cap || (draws && ndraws < next + need)) {
        free(nnew);
        return total == 0 ? BMXG_OK : (n + total > cap ? BMXG_ERR_CAPACITY : BMXG_ERR_ARG);
    }
    const int nreals = SR_first + sp->num_reals, nints = SI_first + sp->num_ints;
    int64_t k = 0;
    for (int64_t i = 0; i < n; ++i) {
        if (!nnew[i]) continue;
        orec_t m = OREC(i), d1 = OREC(n + k), d2 = OREC(n + k + (nnew[i] == 2 ? 1 : 0));
        odraw_t u = {draws, &next, seed, m.id[0], m.id[1], 1};
        for (int c = 0; c < nnew[i]; ++c) {  /* copyChildParameters */
            orec_t *d = c ? &d2 : &d1;
            for (int j = 0; j < nreals; ++j) d->r[j] = m.r[j];
            for (int j = 0; j < nints; ++j) d->q[j] = m.q[j];
        }
        const int id1 = (int)(next_id + k);
        if (nnew[i] == 2) {
            odivide_tip_in_two(sp, &m, &d1, &d2, &u, id1, my_proc, id1 + 1, my_proc);
            d2.id[0] = id1 + 1;
            d2.id[1] = my_proc;
        } else {
            if (m.q[SI_cell_type] == BMXG_YEAST) odivide_cell(sp, &m, &d1, &u);
            else odivide_segment(sp, &m, &d1, &u, id1, my_proc);
            d1.q[SI_id] = id1;
            d1.q[SI_cpu] = my_proc;
        }
        d1.id[0] = id1;
        d1.id[1] = my_proc;
        k += nnew[i];
    }
#undef OREC
    free(nnew);
    return BMXG_OK;
}
