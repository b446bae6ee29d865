// k_rod.cu -- the step for states that hold rod segments (FUNGI), alone or
// mixed with spheres: deterministic bond bookkeeping, the segment-segment
// closest-point contact / bonded-spring force gather with the wall force,
// and the update with the orientation rotation.
//
// Replaces, for FUNGI, the force lambda of src/des/bmx_pc_interaction.cpp:170-279
// with evaluateForce's rod branch (src/chemistry/bmx_cell_interaction_K.H:277-993)
// and evaluateSurfaceForce's rod branch (:1031-1282), and the update lambda
// (bmx_pc_interaction.cpp:311-436) with its orientation rotation (:334-431).
//
// Design notes
//  * The reference edits bond tables from inside its parallel pair loop; its
//    edits of the neighbour j land on a by-value copy (bmx_pc_interaction.cpp:188)
//    and do not persist, so the lasting effect is "each segment repairs its
//    own table".  k_rod_book does exactly that, reading the neighbours'
//    tables as they were at the start of the step (buffer a) and writing the
//    segment's own table to buffer b -- deterministic, and equal to the
//    reference's serial CPU result.
//  * Only segment i's velocity is produced per pair (the j-side accumulation
//    is disabled in the reference, bmx_pc_interaction.cpp:251-261), and the
//    mobility of segment i is linear in its two site forces:
//      vel = 1/2 (Dii + Dij)(f1 + f2),  rot = 1/2 r x (Dii - Dij)(f1 - f2)_perp
//    with Dii = d0 I and Dij = db I + (da - db) n n^T (the rotated tensors of
//    :812-882).  The kernel therefore sums f1 + f2 and f1 - f2 over the pairs
//    and applies the mobility once per segment: the same result up to
//    rounding, without two 3x3 tensor rotations per pair.
//  * FP32F: contact pair math in FP32 on the FP64-differenced bin-relative
//    offsets; pairs whose segments are near-parallel (det < 0.05 Aii Ajj,
//    where the closest-point solve loses precision), pairs whose closest
//    points are within 1 % of the segment lengths (touching or crossing
//    segments, where the separation's direction is end-point rounding noise)
//    and bonded pairs (a spring on the difference of two coincident end
//    points) are done in FP64.
#include "bmxg_stencil.cuh"

namespace bmxg {

namespace {

template <class T>
__device__ __forceinline__ bool in01(T t) { return t >= T(0) && t <= T(1); }

template <class T>
__device__ __forceinline__ T sq3(T a, T b, T c) { return a * a + b * b + c * c; }

// Closest points of segments (a1,a2) and (b1,b2): the case structure of
// evaluateMinimumDistance (bmx_cell_interaction_K.H:51-221), including the
// exact zero tests on Aij and det and the unconstrained result for Aij == 0.
template <class T>
__device__ void min_distance(const T *a1, const T *a2, const T *b1, const T *b2, T &tau_i, T &tau_j)
{
    T ri[3], rj[3], w[3];
    for (int k = 0; k < 3; ++k) {
        ri[k] = a2[k] - a1[k];
        rj[k] = b2[k] - b1[k];
        w[k] = a1[k] - b1[k];
    }
    T rirj = T(0);
    for (int k = 0; k < 3; ++k) rirj += ri[k] * rj[k];
    const T Aii = sq3(ri[0], ri[1], ri[2]);
    const T Ajj = sq3(rj[0], rj[1], rj[2]);
    const T Aij = -rirj;
    const T det = Aii * Ajj - Aij * Aij;
    const T Bi = -(w[0] * ri[0] + w[1] * ri[1] + w[2] * ri[2]);
    const T Bj = w[0] * rj[0] + w[1] * rj[1] + w[2] * rj[2];
    T ti = T(0), tj = T(0);
    bool search = false;
    if (Aij == T(0)) {
        ti = Bi / Aii;
        tj = Bj / Ajj;
    } else if (det == T(0)) {
        const T t0 = Bj / Ajj;
        if (in01(t0)) { ti = T(0); tj = t0; }
        else {
            const T t1 = (Bj + rirj) / Ajj;
            if (in01(t1)) { ti = T(1); tj = t1; }
            else search = true;
        }
    } else {
        ti = (Ajj * Bi - Aij * Bj) / det;
        tj = (Aii * Bj - Aij * Bi) / det;
        if (in01(ti)) {
            if (tj < T(0) || tj > T(1)) {
                const T t0 = Bi / Aii, t1 = (Bi + rirj) / Aii;
                if (in01(t0) && in01(t1)) {
                    const T s0 = sq3(a1[0] + t0 * ri[0] - b1[0], a1[1] + t0 * ri[1] - b1[1],
                                     a1[2] + t0 * ri[2] - b1[2]);
                    const T s1 = sq3(a1[0] + t1 * ri[0] - b2[0], a1[1] + t1 * ri[1] - b2[1],
                                     a1[2] + t1 * ri[2] - b2[2]);
                    if (s0 < s1) { tj = T(0); ti = t0; } else { tj = T(1); ti = t1; }
                } else if (in01(t0)) { tj = T(0); ti = t0; }
                else if (in01(t1)) { tj = T(1); ti = t1; }
                else search = true;
            }
        } else if (in01(tj)) {
            const T t0 = Bj / Ajj, t1 = (Bj + rirj) / Ajj;
            if (in01(t0) && in01(t1)) {
                const T s0 = sq3(b1[0] + t0 * rj[0] - a1[0], b1[1] + t0 * rj[1] - a1[1],
                                 b1[2] + t0 * rj[2] - a1[2]);
                const T s1 = sq3(b1[0] + t1 * rj[0] - a2[0], b1[1] + t1 * rj[1] - a2[1],
                                 b1[2] + t1 * rj[2] - a2[2]);
                if (s0 < s1) { ti = T(0); tj = t0; } else { ti = T(1); tj = t1; }
            } else if (in01(t0)) { ti = T(0); tj = t0; }
            else if (in01(t1)) { ti = T(1); tj = t1; }
            else search = true;
        } else {
            search = true;
        }
    }
    if (search) {
        T m[4];
        m[0] = sq3(a1[0] - b1[0], a1[1] - b1[1], a1[2] - b1[2]);
        m[1] = sq3(a1[0] - b2[0], a1[1] - b2[1], a1[2] - b2[2]);
        m[2] = sq3(a2[0] - b1[0], a2[1] - b1[1], a2[2] - b1[2]);
        m[3] = sq3(a2[0] - b2[0], a2[1] - b2[1], a2[2] - b2[2]);
        int best = 0;
        for (int k = 1; k < 4; ++k)
            if (m[k] < m[best]) best = k;
        ti = (best >= 2) ? T(1) : T(0);
        tj = (best & 1) ? T(1) : T(0);
    }
    tau_i = ti;
    tau_j = tj;
}

// Site forces on segment i from segment j (j's centre at the origin, i's at
// r12): a bonded linear spring between the bonded sites (si, sj in {1,2}),
// otherwise the cubic contact law at the closest points split (1-tau, tau)
// (bmx_cell_interaction_K.H:552-772).  Returns f1 (site 1) and f2 (site 2).
template <class T>
__device__ void rod_site_forces(const T *r12, const T *ni, T Li, const T *nj, T Lj, T rS, T rA, T k,
                                int si, int sj, T kb, T *f1, T *f2, T *r_out = nullptr)
{
    T e1[3], e2[3], g1[3], g2[3];
    for (int d = 0; d < 3; ++d) {
        e1[d] = r12[d] - T(0.5) * ni[d] * Li;
        e2[d] = r12[d] + T(0.5) * ni[d] * Li;
        g1[d] = T(-0.5) * nj[d] * Lj;
        g2[d] = T(0.5) * nj[d] * Lj;
        f1[d] = T(0);
        f2[d] = T(0);
    }
    if ((si == 1 || si == 2) && (sj == 1 || sj == 2)) {
        const T *ea = (si == 1) ? e1 : e2;
        const T *eb = (sj == 1) ? g1 : g2;
        T *f = (si == 1) ? f1 : f2;
        for (int d = 0; d < 3; ++d) f[d] -= kb * (ea[d] - eb[d]);
        return;
    }
    T ti, tj;
    min_distance(e1, e2, g1, g2, ti, tj);
    T dv[3];
    for (int d = 0; d < 3; ++d) dv[d] = (e1[d] + ti * (e2[d] - e1[d])) - (g1[d] + tj * (g2[d] - g1[d]));
    const T r = sqrt(dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2]);
    if (r_out) *r_out = r;
    // r <= 1e-8: the reference keeps the unnormalised separation (its
    // fallback direction goes to shadowing locals, :744-746); so do we.
    if (r > T(1.0e-8)) {
        dv[0] /= r;
        dv[1] /= r;
        dv[2] /= r;
    }
    const T F = (r < rA) ? -k * (r - rA) * (r - rA) * (r - rS) : T(0);
    if (F != T(0)) {
        for (int d = 0; d < 3; ++d) {
            f1[d] += F * dv[d] * (T(1) - ti);
            f2[d] += F * dv[d] * ti;
        }
    }
}

__device__ __forceinline__ int find_in_table(const int *tb, int id, int cpu)
{
    const int nb = min(tb[0], 4);
    for (int k = 0; k < nb; ++k)
        if (tb[1 + k] == id && tb[5 + k] == cpu) return k;
    return -1;
}

// The site of the first entry of a register-held table tb (n_bnds, ids[4],
// cpus[4], sites[4]) that names (id, cpu), or 0: the same answer as
// tb[9 + find_in_table(...)], by selects over constant indices so the table
// never goes to local memory.
__device__ __forceinline__ int table_site(const int *tb, int id, int cpu)
{
    const int nb = min(tb[0], 4);
    int site = 0;
#pragma unroll
    for (int k = 3; k >= 0; --k)
        if (k < nb && tb[1 + k] == id && tb[5 + k] == cpu) site = tb[9 + k];
    return site;
}

__device__ __forceinline__ int find_in_plane_table(const int *tab, int n, int j, int id, int cpu)
{
    const int nb = min(__ldg(&tab[j]), 4);
    for (int k = 0; k < nb; ++k)
        if (__ldg(&tab[(size_t)(1 + k) * n + j]) == id && __ldg(&tab[(size_t)(5 + k) * n + j]) == cpu) return k;
    return -1;
}

// exact FP64 separation of slot i from the (image of) slot j, as the
// reference's loop computes it (bmx_pc_interaction.cpp:191-197)
__device__ __forceinline__ double sep64(const DevState &S, const DevGeom &G, int a, int j, int sx, int sy,
                                        double xi, double yi, double zi, double *d)
{
    const double xj = sx ? S.x[a][j] + (double)sx * G.len[0] : S.x[a][j];
    const double yj = sy ? S.y[a][j] + (double)sy * G.len[1] : S.y[a][j];
    d[0] = xi - xj;
    d[1] = yi - yj;
    d[2] = zi - S.z[a][j];
    return d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
}

// The interaction gate r^2 <= (r_lm - 1e-15)^2 (and BMXCheckPair's
// r^2 <= neighborhood) decided from the FP32 bin offsets where they settle it:
// the offsets are the FP64 differences rounded once, so the FP32 separation
// is within ~1e-9 cm of the exact one, and a pair more than 1e-5 r_lm from
// the gate is decided without FP64 arithmetic; the others take the exact
// FP64 test.  Returns the decision and the FP32 separation r12f.
__device__ __forceinline__ bool rod_gate(const DevState &S, const DevGeom &G, const DevParams &P, int a, int j,
                                         int dxs, int dys, int dzs, int sx, int sy, float4 me, float Lif, float Ljf,
                                         double xi, double yi, double zi, double Li, float *r12f)
{
    const float4 q = __ldg(&S.rel[a][j]);
    r12f[0] = (me.x - q.x) - (float)dxs * G.dxf[0];
    r12f[1] = (me.y - q.y) - (float)dys * G.dxf[1];
    r12f[2] = (me.z - q.z) - (float)dzs * G.dxf[2];
    const float r2f = r12f[0] * r12f[0] + r12f[1] * r12f[1] + r12f[2] * r12f[2];
    if (G.nbh_trivial) {
        const float rlmf = 1.5f * (Lif + Ljf) + P.bw32;
        const float lo = rlmf * (1.0f - 1.0e-5f), hi = rlmf * (1.0f + 1.0e-5f);
        if (r2f <= lo * lo) return true;
        if (r2f > hi * hi) return false;
    }
    double d[3];
    const double r2 = sep64(S, G, a, j, sx, sy, xi, yi, zi, d);
    if (!G.nbh_trivial && !(r2 <= P.nbh)) return false;
    const double rlm = 1.5 * (Li + S.clen[j]) + P.bw;
    return r2 <= (rlm - kSmall) * (rlm - kSmall);
}

// ---- bookkeeping ----------------------------------------------------------
// LIST: also record the segment's gated pairs, in the order of its walk, for
// the FP32F pipeline (rnb, rcnt; the step's largest count into rctl->kmax).
template <bool LIST>
__global__ void k_rod_book(const DevState S, const DevParams P, int a)
{
    const int b = a ^ 1;
    const int n = S.n;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int cnt = 0;
        S.fflag[i] = 0;  // flag resets of bmx_pc_interaction.cpp:178-180
        S.sflag[i] = 0;
        S.nflag[i] = 0;
        int tb[13];
        for (int k = 0; k < 13; ++k) tb[k] = S.tab[a][(size_t)k * n + i];
        {   // this step's FP32 axis and length, for the FP32F force kernel
            const double4_32a tr = S.trig[a][i];
            S.axf[i] = make_float4(d2f_rn(tr.y * tr.z), d2f_rn(tr.y * tr.w), d2f_rn(tr.x), d2f_rn(S.clen[i]));
        }
        if (S.ctype[i] == kFungi) {
            const DevGeom &G = geom_of(S, i);
            int bx, by;
            col_to_bxy(G, S.col[a][i], bx, by);
            const double xi = S.x[a][i], yi = S.y[a][i], zi = S.z[a][i];
            const double Li = S.clen[i];
            const float Lif = d2f_rn(Li);
            const float4 me = S.rel[a][i];
            const int iid = S.id[i], icpu = S.cpu[i];
            const int fs = S.fix_site[i];
            int pos = S.position[i];
            bool any = false;
            int rep = 0;
            visit_stencil(S, G, a, i, bx, by, S.iz[a][i], [&](int j, int dxs, int dys, int dzs, int sx, int sy) {
                if (S.ctype[j] != kFungi) return;
                float r12f[3];
                if (!rod_gate(S, G, P, a, j, dxs, dys, dzs, sx, sy, me, Lif, d2f_rn(S.clen[j]), xi, yi, zi, Li, r12f))
                    return;
                any = true;
                if (LIST) {
                    if (cnt < kRodCap) {
                        const int code = ((dxs + 1) * 9 + (dys + 1) * 3 + (dzs + 1)) | (((sx + 1) * 3 + (sy + 1)) << 5);
                        S.rnb[(size_t)cnt * n + i] = make_int2(j, code);
                    }
                    ++cnt;
                }
                const int jid = S.id[j], jcpu = S.cpu[j];
                // position fix-up (bmx_cell_interaction_K.H:338-362); the
                // neighbour's position is only tested against TIP, which no
                // thread writes, so reading it while others update theirs is safe
                if (pos == kSecond1 || pos == kSecond2) {
                    const int site = (pos == kSecond1) ? 1 : 2;
                    const int nb = min(tb[0], 4);
                    int k = 0;
                    for (; k < nb; ++k)
                        if (tb[1 + k] == jid && tb[5 + k] == jcpu && tb[9 + k] == site) break;
                    if (k < nb && S.position[j] != kTip) pos = kInterior;
                }
                // half-bond repair of i (:370-467)
                const bool i_to_j = find_in_table(tb, jid, jcpu) >= 0;
                const bool j_to_i = find_in_plane_table(S.tab[a], n, j, iid, icpu) >= 0;
                if (!i_to_j && j_to_i) {
                    const int nb = tb[0];
                    if (nb >= 0 && nb < 4) {
                        const int isite = (fs == 0) ? (tb[9] == 1 ? 2 : 1) : fs;
                        tb[1 + nb] = jid;
                        tb[5 + nb] = jcpu;
                        tb[9 + nb] = isite;
                        tb[0] = nb + 1;
                        ++rep;
                    }
                }
            });
            S.position[i] = pos;
            if (any)
                for (int k = 0; k < 6; ++k) S.dltd[(size_t)k * n + i] = -1;
            if (rep) atomicAdd(&S.cnt->bond_repairs, (unsigned long long)rep);
        }
        for (int k = 0; k < 13; ++k) S.tab[b][(size_t)k * n + i] = tb[k];
        if (LIST) {
            // the site of i that its repaired table bonds to each recorded
            // neighbour (1 or 2, else 0) into bits 9-10
            for (int k = 0; k < min(cnt, kRodCap); ++k) {
                int2 &e = S.rnb[(size_t)k * n + i];
                const int site = table_site(tb, S.id[e.x], S.cpu[e.x]);
                e.y |= ((site == 1 || site == 2) ? site : 0) << 9;
            }
            S.rcnt[i] = cnt;
            const unsigned m = __activemask();
            const int w = __reduce_max_sync(m, min(cnt, kRodCap));
            if ((threadIdx.x & 31) == __ffs(m) - 1 && w > 0) atomicMax(&S.rctl->kmax, w);
        }
    }
}

// ---- per-segment mobility -----------------------------------------------------
// Mobility of a segment from its area, length and the viscosity
// (bmx_cell_interaction_K.H:812-840): d0 for the segment as a sphere of the
// same area, da along and db across its axis.  Stored as the combinations the
// force gather applies, (d0 + db, da - db, (d0 - db) / 2), each the FP64
// expression the gather evaluated per step before; none of the inputs changes
// during a step, so it runs when a state or the parameters load.
__global__ void k_rod_mobility(const DevState S, const DevParams P)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < S.n; i += gridDim.x * blockDim.x) {
        double4_32a m = make_trig(0.0, 0.0, 0.0, 0.0);
        if (S.ctype[i] == kFungi) {
            const double Li = S.clen[i];
            const double area = S.area[i] / 2.0;
            const double arad = sqrt(area / (4.0 * kPi));
            const double d0 = 1.0 / (6.0 * kPi * arad * P.visc);
            double da, db;
            if (Li > 2.0 * arad) {
                da = (Li * Li - 2.0 * arad * arad / 3.0) / (4.0 * kPi * pow(Li, 3.0) * P.visc);
                db = (Li * Li + 2.0 * arad * arad / 3.0) / (8.0 * kPi * pow(Li, 3.0) * P.visc);
            } else {
                da = (1.0 - 3.0 * Li / (16.0 * arad)) / (6.0 * kPi * arad * P.visc);
                db = (1.0 - 9.0 * Li / (32.0 * arad)) / (6.0 * kPi * arad * P.visc);
            }
            m = make_trig(d0 + db, da - db, 0.5 * (d0 - db), 0.0);
        }
        S.mob[i] = m;
    }
}

// Velocity (acc[0..2]) and rotation (acc[3..5]) of a segment in FP32 from its
// site-force sums Sv = sum f1 + f2 and Dv = sum f1 - f2, its mobility m and
// the growth-surface force on its two sites (bmx_cell_interaction_K.H:812-882,
// :1067-1281), the axis from ni and L instead of the difference of the two
// site positions (which FP32 would round at the magnitude of the position);
// dzc = centre height above the surface, rounded once from FP64.
__device__ __forceinline__ void rod_velocity32(const float *ni, float L, const float *Sv, const float *Dv,
                                               const double4_32a &m, float dzc, float rS, const DevParams &P,
                                               float *acc)
{
    const float m0 = d2f_rn(m.x), m1 = d2f_rn(m.y), m2 = d2f_rn(m.z);
    const float ns = ni[0] * Sv[0] + ni[1] * Sv[1] + ni[2] * Sv[2];
    float ax[3];
    for (int k = 0; k < 3; ++k) {
        acc[k] = 0.5f * (m0 * Sv[k] + m1 * ns * ni[k]);
        ax[k] = -ni[k] * L;  // site 1 minus site 2
    }
    acc[3] = m2 * (ax[1] * Dv[2] - ax[2] * Dv[1]);
    acc[4] = m2 * (ax[2] * Dv[0] - ax[0] * Dv[2]);
    acc[5] = m2 * (ax[0] * Dv[1] - ax[1] * Dv[0]);
    const float h = 0.5f * ni[2] * L;
    float w1[3] = {0.0f, 0.0f, wall_law32(dzc - h, rS, P.z_k32, P.z_bw32, P.z_g32)};
    float w2[3] = {0.0f, 0.0f, wall_law32(dzc + h, rS, P.z_k32, P.z_bw32, P.z_g32)};
    const float ra = sqrtf(ax[0] * ax[0] + ax[1] * ax[1] + ax[2] * ax[2]);
    const float un[3] = {ax[0] / ra, ax[1] / ra, ax[2] / ra};
    const float fn = (w1[2] - w2[2]) * un[2];
    float vw[3];
    for (int k = 0; k < 3; ++k) {
        w1[k] -= 0.5f * fn * un[k];
        w2[k] += 0.5f * fn * un[k];
        vw[k] = 0.5f * (w1[k] + w2[k]);
    }
    for (int k = 0; k < 3; ++k) {
        w1[k] -= 0.5f * vw[k];
        w2[k] -= 0.5f * vw[k];
    }
    acc[0] += vw[0];
    acc[1] += vw[1];
    acc[2] += vw[2];
    acc[3] += 0.5f * ((ax[1] * w1[2] - ax[2] * w1[1]) - (ax[1] * w2[2] - ax[2] * w2[1]));
    acc[4] += 0.5f * ((ax[2] * w1[0] - ax[0] * w1[2]) - (ax[2] * w2[0] - ax[0] * w2[2]));
    acc[5] += 0.5f * ((ax[0] * w1[1] - ax[1] * w1[0]) - (ax[0] * w2[1] - ax[1] * w2[0]));
}

// ---- force gather ----------------------------------------------------------
// The force gather of slot i by a walk of its stencil (fc, fix_site).
template <int PREC>
__device__ __forceinline__ void rod_force_slot(const DevState &S, const DevParams &P, int a, int i)
{
    const int b = a ^ 1;
    const int n = S.n;
    {
        const DevGeom &G = geom_of(S, i);
        int bx, by;
        col_to_bxy(G, S.col[a][i], bx, by);
        const int izi = S.iz[a][i];
        const double xi = S.x[a][i], yi = S.y[a][i], zi = S.z[a][i];
        const double ri = S.rad[i];
        const int ti = S.ctype[i];
        double acc[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        if (ti == kYeast) {
            visit_stencil(S, G, a, i, bx, by, izi, [&](int j, int, int, int, int sx, int sy) {
                if (S.ctype[j] != kYeast) return;  // mixed pairs: no force (cutoff 0)
                double d[3];
                const double r2 = sep64(S, G, a, j, sx, sy, xi, yi, zi, d);
                if (!G.nbh_trivial && !(r2 <= P.nbh)) return;
                const double rj = S.rad[j];
                const double rlm = ri + rj + P.bw;
                if (!(r2 <= (rlm - kSmall) * (rlm - kSmall))) return;
                const double rS = ri + rj, rA = rS + P.bw;
                const double rn = sqrt(r2);
                const double ux = d[0] / rn, uy = d[1] / rn, uz = d[2] / rn;
                const double F = (rn < rA) ? -P.k * (rn - rA) * (rn - rA) * (rn - rS) : 0.0;
                acc[0] += F * ux;
                acc[1] += F * uy;
                acc[2] += F * uz;
            });
            acc[2] += wall_law(zi, ri, P);
        } else if (ti == kFungi) {
            const double Li = S.clen[i];
            const double4_32a tri = S.trig[a][i];  // (ct, st, cp, sp)
            const double ni[3] = {tri.y * tri.z, tri.y * tri.w, tri.x};
            const int iid = S.id[i], icpu = S.cpu[i];
            const int itip = S.fuse_tip[i];
            const double bsi = S.bscale[i];
            int tb[13];
#pragma unroll
            for (int k = 0; k < 13; ++k) tb[k] = S.tab[b][(size_t)k * n + i];
            const float4 me = S.rel[a][i];
            const float4 axi = S.axf[i];  // FP32 axis and length (k_rod_book)
            double Sv[3] = {0.0, 0.0, 0.0}, Dv[3] = {0.0, 0.0, 0.0};
            float Svf[3] = {0.0f, 0.0f, 0.0f}, Dvf[3] = {0.0f, 0.0f, 0.0f};  // the FP32F pairs' sums
            visit_stencil(S, G, a, i, bx, by, izi, [&](int j, int dxs, int dys, int dzs, int sx, int sy) {
                if (S.ctype[j] != kFungi) return;
                const float4 axj = __ldg(&S.axf[j]);
                float r12f[3];
                if (!rod_gate(S, G, P, a, j, dxs, dys, dzs, sx, sy, me, axi.w, axj.w, xi, yi, zi, Li, r12f)) return;
                // bonds: mutual entries in both (repaired) tables
                int si = 0, sj = 0;
                double kb = P.k_bond;
                const int isite = table_site(tb, S.id[j], S.cpu[j]);
                if (isite != 0) {  // (an entry of site 0 bonds nothing either way)
                    const int jb = find_in_plane_table(S.tab[b], n, j, iid, icpu);
                    if (jb >= 0) {
                        si = isite;
                        sj = __ldg(&S.tab[b][(size_t)(9 + jb) * n + j]);
                        const int jtip = S.fuse_tip[j];
                        if ((itip > 0 && itip == si) || (jtip > 0 && jtip == sj)) kb = bsi * S.bscale[j] * kb;
                    }
                }
                if (PREC == BMXG_FP32F_FORM) {
                    // the pair in FP32 from the bin offsets and this step's FP32 axes,
                    // except: bonded pairs (their spring acts on the difference of
                    // two coincident end points, which FP32 end points would swamp
                    // with rounding noise: k_bond x ulp of the segment length),
                    // near-parallel segments (det < 0.05 Aii Ajj of the closest-point
                    // system: the FP64 solve) and touching or crossing segments
                    // (closest points within 1 % of the lengths: the direction of an
                    // FP32 separation is end-point rounding noise there)
                    const float nif[3] = {axi.x, axi.y, axi.z};
                    const float njf[3] = {axj.x, axj.y, axj.z};
                    const float rij = nif[0] * njf[0] + nif[1] * njf[1] + nif[2] * njf[2];
                    const bool bonded = (si == 1 || si == 2) && (sj == 1 || sj == 2);
                    if (!bonded && 1.0f - rij * rij >= 0.05f) {
                        const float rSf = me.w + __ldg(&S.rel[a][j]).w;
                        float g1[3], g2[3], rf;
                        // (not bonded: the spring constant is not used)
                        rod_site_forces<float>(r12f, nif, axi.w, njf, axj.w, rSf, rSf + P.bw32, P.k32, si, sj,
                                               0.0f, g1, g2, &rf);
                        if (rf >= 0.01f * (axi.w + axj.w)) {
                            for (int k = 0; k < 3; ++k) {
                                Svf[k] += g1[k] + g2[k];
                                Dvf[k] += g1[k] - g2[k];
                            }
                            return;
                        }
                    }
                }
                double d[3];
                sep64(S, G, a, j, sx, sy, xi, yi, zi, d);
                const double4_32a trj = S.trig[a][j];
                const double rS = ri + S.rad[j];
                const double rA = rS + P.bw;
                const double nj[3] = {trj.y * trj.z, trj.y * trj.w, trj.x};
                double f1[3], f2[3];
                rod_site_forces<double>(d, ni, Li, nj, S.clen[j], rS, rA, P.k, si, sj, kb, f1, f2);
                for (int k = 0; k < 3; ++k) {
                    Sv[k] += f1[k] + f2[k];
                    Dv[k] += f1[k] - f2[k];
                }
            });
            // mobility of segment i (bmx_cell_interaction_K.H:812-840), k_rod_mobility
            const double4_32a mb = S.mob[i];
            if (PREC == BMXG_FP32F_FORM) {
                // the FP64 pairs' sums plus the FP32 pairs' (exactly converted), rounded
                // once; velocity, rotation and the surface force in FP32
                float sv[3], dv[3], af[6];
                for (int k = 0; k < 3; ++k) {
                    sv[k] = d2f_rn(Sv[k] + f2d_int(Svf[k]));
                    dv[k] = d2f_rn(Dv[k] + f2d_int(Dvf[k]));
                }
                const float nif[3] = {axi.x, axi.y, axi.z};
                rod_velocity32(nif, axi.w, sv, dv, mb, d2f_rn(zi - P.z_wall), me.w, P, af);
                for (int k = 0; k < 6; ++k) acc[k] = f2d_int(af[k]);
                S.fix_site[i] = 0;  // evaluateSurfaceForce (bmx_cell_interaction_K.H:1060)
                for (int c = 0; c < 6; ++c) S.fc[(size_t)c * n + i] = acc[c];
                return;
            }
            const double ns = ni[0] * Sv[0] + ni[1] * Sv[1] + ni[2] * Sv[2];
            double rv[3];
            for (int k = 0; k < 3; ++k) {
                acc[k] = 0.5 * (mb.x * Sv[k] + mb.y * ns * ni[k]);
                rv[k] = (-0.5 * ni[k] * Li) - (0.5 * ni[k] * Li);  // site 1 minus site 2
            }
            const double c = mb.z;
            acc[3] = c * (rv[1] * Dv[2] - rv[2] * Dv[1]);
            acc[4] = c * (rv[2] * Dv[0] - rv[0] * Dv[2]);
            acc[5] = c * (rv[0] * Dv[1] - rv[1] * Dv[0]);
            // growth-surface force on both sites (bmx_cell_interaction_K.H:1067-1281;
            // its mobility block :1176-1265 is overwritten there and has no effect)
            double u1[3], u2[3], ax[3];
            const double pc[3] = {xi, yi, zi};
            for (int k = 0; k < 3; ++k) {
                u1[k] = pc[k] - 0.5 * ni[k] * Li;
                u2[k] = pc[k] + 0.5 * ni[k] * Li;
                ax[k] = u1[k] - u2[k];
            }
            double w1[3] = {0.0, 0.0, wall_law(u1[2], ri, P)};
            double w2[3] = {0.0, 0.0, wall_law(u2[2], ri, P)};
            const double ra = sqrt(ax[0] * ax[0] + ax[1] * ax[1] + ax[2] * ax[2]);
            const double un[3] = {ax[0] / ra, ax[1] / ra, ax[2] / ra};
            const double fn = (w1[0] - w2[0]) * un[0] + (w1[1] - w2[1]) * un[1] + (w1[2] - w2[2]) * un[2];
            double vw[3];
            for (int k = 0; k < 3; ++k) {
                w1[k] -= 0.5 * fn * un[k];
                w2[k] += 0.5 * fn * un[k];
            }
            for (int k = 0; k < 3; ++k) vw[k] = 0.5 * (w1[k] + w2[k]);
            for (int k = 0; k < 3; ++k) {
                w1[k] -= 0.5 * vw[k];
                w2[k] -= 0.5 * vw[k];
            }
            double rw[3];
            rw[0] = 0.5 * (ax[1] * w1[2] - ax[2] * w1[1]);
            rw[1] = 0.5 * (ax[2] * w1[0] - ax[0] * w1[2]);
            rw[2] = 0.5 * (ax[0] * w1[1] - ax[1] * w1[0]);
            rw[0] += -0.5 * (ax[1] * w2[2] - ax[2] * w2[1]);
            rw[1] += -0.5 * (ax[2] * w2[0] - ax[0] * w2[2]);
            rw[2] += -0.5 * (ax[0] * w2[1] - ax[1] * w2[0]);
            for (int k = 0; k < 3; ++k) {
                acc[k] += vw[k];
                acc[3 + k] += rw[k];
            }
            S.fix_site[i] = 0;  // evaluateSurfaceForce (:1060)
        }
        for (int c = 0; c < 6; ++c) S.fc[(size_t)c * n + i] = acc[c];
    }
}

template <int PREC>
__global__ void __launch_bounds__(128) k_rod_force(const DevState S, const DevParams P, int a)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < S.n; i += gridDim.x * blockDim.x)
        rod_force_slot<PREC>(S, P, a, i);
}

// ---- FP32F pipeline ---------------------------------------------------------
// With every segment's gated pairs recorded by k_rod_book, the FP32F force
// gather runs flat instead of one stencil walk per thread (whose lanes
// diverge over pair counts and over the FP32 and FP64 paths):
//   k_rod_pair32  one pair per thread (pair k of segment i); evaluates it in
//                 FP32 where the FP32F form allows, else queues it;
//   k_rod_pair64  the queued pairs, one per thread, in FP64 (full warps on
//                 the FP64 pipe);
//   k_rod_seg32   per segment: its pairs' f1 + f2 and f1 - f2 summed in FP64 in
//                 list order, then mobility and surface force in FP32.
// Each pair writes its own slot, so the sums do not depend on the order in
// which the queue filled.

__device__ __forceinline__ void decode_pair(int code, int &dxs, int &dys, int &dzs, int &sx, int &sy)
{
    const int c = code & 31, s = (code >> 5) & 15;
    dxs = c / 9 - 1;
    dys = (c / 3) % 3 - 1;
    dzs = c % 3 - 1;
    sx = s / 3 - 1;
    sy = s % 3 - 1;
}

__device__ __forceinline__ void put_pair(const DevState &S, int i, int k, const double *sv, const double *dv)
{
    const size_t n = (size_t)S.n;
    for (int c = 0; c < 3; ++c) {
        S.rres[((size_t)c * kRodCap + k) * n + i] = sv[c];
        S.rres[((size_t)(3 + c) * kRodCap + k) * n + i] = dv[c];
    }
}

__global__ void __launch_bounds__(256) k_rod_pair32(const DevState S, const DevParams P, int a)
{
    const int b = a ^ 1;
    const int n = S.n;
    const long long total = (long long)n * S.rctl->kmax;
    const int lane = threadIdx.x & 31;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(t / n);
        const int i = (int)(t - (long long)k * n);
        bool q64 = false;
        int si = 0, sj = 0;
        if (k < S.rcnt[i]) {
            const int2 e = S.rnb[(size_t)k * n + i];
            const int j = e.x;
            int dxs, dys, dzs, sx, sy;
            decode_pair(e.y, dxs, dys, dzs, sx, sy);
            const DevGeom &G = geom_of(S, i);
            const float4 me = S.rel[a][i], q = __ldg(&S.rel[a][j]);
            // the offsets of the gate (rod_gate), recomputed
            float r12f[3] = {(me.x - q.x) - (float)dxs * G.dxf[0], (me.y - q.y) - (float)dys * G.dxf[1],
                             (me.z - q.z) - (float)dzs * G.dxf[2]};
            // bonded: i's repaired table names j (the site k_rod_book found) and
            // j's names i
            const int isite = (e.y >> 9) & 3;
            if (isite) {
                const int jb = find_in_plane_table(S.tab[b], n, j, S.id[i], S.cpu[i]);
                if (jb >= 0) {
                    const int s2 = __ldg(&S.tab[b][(size_t)(9 + jb) * n + j]);
                    si = isite;
                    sj = (s2 == 1 || s2 == 2) ? s2 : 0;
                }
            }
            // FP32 unless bonded, near-parallel or touching (as rod_force_slot)
            q64 = true;
            const float4 axi = S.axf[i], axj = __ldg(&S.axf[j]);
            const float nif[3] = {axi.x, axi.y, axi.z};
            const float njf[3] = {axj.x, axj.y, axj.z};
            const float rij = nif[0] * njf[0] + nif[1] * njf[1] + nif[2] * njf[2];
            if (!(si && sj) && 1.0f - rij * rij >= 0.05f) {
                const float rSf = me.w + q.w;
                float g1[3], g2[3], rf;
                rod_site_forces<float>(r12f, nif, axi.w, njf, axj.w, rSf, rSf + P.bw32, P.k32, 0, 0, 0.0f, g1, g2,
                                       &rf);
                if (rf >= 0.01f * (axi.w + axj.w)) {
                    double sv[3], dv[3];
                    for (int c = 0; c < 3; ++c) {
                        sv[c] = f2d_int(g1[c] + g2[c]);
                        dv[c] = f2d_int(g1[c] - g2[c]);
                    }
                    put_pair(S, i, k, sv, dv);
                    q64 = false;
                }
            }
        }
        // queue the FP64 pairs, one atomic per warp
        const unsigned am = __activemask();
        const unsigned qm = __ballot_sync(am, q64);
        if (qm) {
            const int leader = __ffs(qm) - 1;
            int base = 0;
            if (lane == leader) base = atomicAdd(&S.rctl->nwork, __popc(qm));
            base = __shfl_sync(am, base, leader);
            if (q64) S.rwork[base + __popc(qm & ((1u << lane) - 1u))] = make_int2(i, k | (si << 8) | (sj << 12));
        }
    }
}

__global__ void __launch_bounds__(128) k_rod_pair64(const DevState S, const DevParams P, int a)
{
    const int n = S.n;
    const int nw = S.rctl->nwork;
    for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < nw; w += gridDim.x * blockDim.x) {
        const int2 it = S.rwork[w];
        const int i = it.x, k = it.y & 255, si = (it.y >> 8) & 15, sj = (it.y >> 12) & 15;
        const int2 e = S.rnb[(size_t)k * n + i];
        const int j = e.x;
        int dxs, dys, dzs, sx, sy;
        decode_pair(e.y, dxs, dys, dzs, sx, sy);
        const DevGeom &G = geom_of(S, i);
        double kb = P.k_bond;
        if (si && sj) {  // fusing tips (bmx_cell_interaction_K.H:552-600)
            const int itip = S.fuse_tip[i], jtip = S.fuse_tip[j];
            if ((itip > 0 && itip == si) || (jtip > 0 && jtip == sj)) kb = S.bscale[i] * S.bscale[j] * kb;
        }
        double d[3];
        sep64(S, G, a, j, sx, sy, S.x[a][i], S.y[a][i], S.z[a][i], d);
        const double4_32a tri = S.trig[a][i], trj = S.trig[a][j];
        const double ni[3] = {tri.y * tri.z, tri.y * tri.w, tri.x};
        const double nj[3] = {trj.y * trj.z, trj.y * trj.w, trj.x};
        const double rS = S.rad[i] + S.rad[j];
        const double rA = rS + P.bw;
        double f1[3], f2[3], sv[3], dv[3];
        rod_site_forces<double>(d, ni, S.clen[i], nj, S.clen[j], rS, rA, P.k, si, sj, kb, f1, f2);
        for (int c = 0; c < 3; ++c) {
            sv[c] = f1[c] + f2[c];
            dv[c] = f1[c] - f2[c];
        }
        put_pair(S, i, k, sv, dv);
    }
}

__global__ void __launch_bounds__(128) k_rod_seg32(const DevState S, const DevParams P, int a)
{
    const int n = S.n;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int cnt = S.rcnt[i];
        if (S.ctype[i] != kFungi || cnt > kRodCap) {
            // spheres of a mixed state, and a segment with more pairs than the
            // lists hold: the walk
            rod_force_slot<BMXG_FP32F_FORM>(S, P, a, i);
            continue;
        }
        double Sv[3] = {0.0, 0.0, 0.0}, Dv[3] = {0.0, 0.0, 0.0};
        for (int k = 0; k < cnt; ++k)
            for (int c = 0; c < 3; ++c) {
                Sv[c] += S.rres[((size_t)c * kRodCap + k) * n + i];
                Dv[c] += S.rres[((size_t)(3 + c) * kRodCap + k) * n + i];
            }
        const float4 axi = S.axf[i];
        float sv[3], dv[3], af[6];
        for (int c = 0; c < 3; ++c) {
            sv[c] = d2f_rn(Sv[c]);
            dv[c] = d2f_rn(Dv[c]);
        }
        const float nif[3] = {axi.x, axi.y, axi.z};
        rod_velocity32(nif, axi.w, sv, dv, S.mob[i], d2f_rn(S.z[a][i] - P.z_wall), S.rel[a][i].w, P, af);
        for (int c = 0; c < 6; ++c) S.fc[(size_t)c * n + i] = f2d_int(af[c]);
        S.fix_site[i] = 0;  // evaluateSurfaceForce (bmx_cell_interaction_K.H:1060)
    }
}

// ---- update ---------------------------------------------------------------
__global__ void k_rod_update(const DevState S, double dt, int a)
{
    const int b = a ^ 1;
    const int n = S.n;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const DevGeom &G = geom_of(S, i);
        const double v[3] = {S.fc[i], S.fc[(size_t)n + i], S.fc[(size_t)2 * n + i]};
        const double w[3] = {S.fc[(size_t)3 * n + i], S.fc[(size_t)4 * n + i], S.fc[(size_t)5 * n + i]};
        S.vx[i] = v[0];
        S.vy[i] = v[1];
        S.vz[i] = v[2];
        S.wx[i] = w[0];
        S.wy[i] = w[1];
        S.wz[i] = w[2];
        double nx = S.x[a][i] + dt * v[0];
        double ny = S.y[a][i] + dt * v[1];
        const double nz = S.z[a][i] + dt * v[2];
        double th = S.theta[a][i], ph = S.phi[a][i];
        double4_32a tr = S.trig[a][i];
        if (S.ctype[i] == kFungi) {
            // rotate the axis by |omega| dt (bmx_pc_interaction.cpp:334-431)
            const double ct = tr.x, st = tr.y, cp = tr.z, sp = tr.w;
            const double R[3][3] = {{cp * st, -sp, -cp * ct}, {sp * st, cp, -sp * ct}, {ct, 0.0, st}};
            double om[3];
            for (int r = 0; r < 3; ++r) {
                om[r] = 0.0;
                for (int c = 0; c < 3; ++c) om[r] += R[c][r] * w[c];
            }
            const double L = S.clen[i];
            om[0] = 0.0;
            om[1] *= 2.0 / (L * L);
            om[2] *= 2.0 / (L * L);
            double on = sqrt(om[1] * om[1] + om[2] * om[2]);
            if (on > 0.0) {
                om[1] /= on;
                om[2] /= on;
            }
            const double c = om[2], s = om[1];
            const double Q[3][3] = {{1.0, 0.0, 0.0}, {0.0, c, -s}, {0.0, s, c}};
            const double ang = on * dt;
            double sa, ca;
            sincos(ang, &sa, &ca);  // one argument reduction for both
            const double u[3] = {ca, sa, 0.0};
            double q[3], nd[3];
            for (int r = 0; r < 3; ++r) {
                q[r] = 0.0;
                for (int cc = 0; cc < 3; ++cc) q[r] += Q[cc][r] * u[cc];
            }
            for (int r = 0; r < 3; ++r) {
                nd[r] = 0.0;
                for (int cc = 0; cc < 3; ++cc) nd[r] += R[r][cc] * q[cc];
            }
            th = acos(nd[2]);
            const double rho = sqrt(nd[0] * nd[0] + nd[1] * nd[1]);
            if (rho > 0.0) nd[0] /= rho;
            ph = acos(nd[0]);
            if (nd[1] < 0.0) ph = 2.0 * kPi - ph;
            double st2, ct2, sp2, cp2;
            sincos(th, &st2, &ct2);
            sincos(ph, &sp2, &cp2);
            tr = make_trig(ct2, st2, cp2, sp2);
        }
        S.theta[b][i] = th;
        S.phi[b][i] = ph;
        S.trig[b][i] = tr;
        if (G.per[0]) nx = wrap1(nx, G.plo[0], G.phi[0], G.len[0]);
        if (G.per[1]) ny = wrap1(ny, G.plo[1], G.phi[1], G.len[1]);
        S.x[b][i] = nx;
        S.y[b][i] = ny;
        S.z[b][i] = nz;
        rebin_slot(S, G, i, nx, ny, nz, S.rad[i], b);
    }
}

// ---- InitBonds ---------------------------------------------------------------
// Start-up bond detection (bmx_pc_interaction.cpp:500-626 with fixBonds,
// bmx_cell_interaction_K.H:1287-1440): for every listed FUNGI-FUNGI pair
// within the interaction gate, the four end pairs (i1,j1), (i2,j1), (i1,j2),
// (i2,j2) are tried in that order and the first closer than rlim appends
// (id_j, cpu_j, site of i) to i's table.  As in the force gather, the
// neighbour is a copy, so only i's own table changes; each thread owns its
// row and appends in the reference's list order.  A fifth bond (past the
// reference's four table slots) is counted, not written.
__global__ void k_init_bonds(const DevState S, const DevParams P, int a, double rlim,
                             unsigned long long *counts)
{
    const int n = S.n;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (S.ctype[i] != kFungi) continue;
        const DevGeom &G = geom_of(S, i);
        int bx, by;
        col_to_bxy(G, S.col[a][i], bx, by);
        const double xi = S.x[a][i], yi = S.y[a][i], zi = S.z[a][i];
        const double Li = S.clen[i];
        const double4_32a tri = S.trig[a][i];
        const double ni[3] = {tri.y * tri.z, tri.y * tri.w, tri.x};
        int nb = S.tab[a][i];
        unsigned long long add = 0, over = 0;
        visit_stencil(S, G, a, i, bx, by, S.iz[a][i], [&](int j, int, int, int, int sx, int sy) {
            if (S.ctype[j] != kFungi) return;
            double d[3];
            const double r2 = sep64(S, G, a, j, sx, sy, xi, yi, zi, d);
            if (!G.nbh_trivial && !(r2 <= P.nbh)) return;
            const double Lj = S.clen[j];
            const double rlm = 1.5 * (Li + Lj) + P.bw;
            if (!(r2 <= (rlm - kSmall) * (rlm - kSmall))) return;
            const double4_32a trj = S.trig[a][j];
            const double nj[3] = {trj.y * trj.z, trj.y * trj.w, trj.x};
            double e[4][3];  // i1, i2, j1, j2 with j's centre at the origin
            for (int k = 0; k < 3; ++k) {
                e[0][k] = d[k] - 0.5 * ni[k] * Li;
                e[1][k] = d[k] + 0.5 * ni[k] * Li;
                e[2][k] = -0.5 * nj[k] * Lj;
                e[3][k] = 0.5 * nj[k] * Lj;
            }
            for (int m = 0; m < 4; ++m) {
                const int si = (m & 1) + 1, sj = (m >> 1) + 1;  // (1,1) (2,1) (1,2) (2,2)
                const double *p = e[si - 1], *q = e[1 + sj];
                const double rx = p[0] - q[0], ry = p[1] - q[1], rz = p[2] - q[2];
                if (sqrt(rx * rx + ry * ry + rz * rz) < rlim) {
                    if (nb >= 0 && nb < 4) {
                        S.tab[a][(size_t)(1 + nb) * n + i] = S.id[j];
                        S.tab[a][(size_t)(5 + nb) * n + i] = S.cpu[j];
                        S.tab[a][(size_t)(9 + nb) * n + i] = si;
                        ++nb;
                        ++add;
                    } else {
                        ++over;
                    }
                    break;
                }
            }
        });
        S.tab[a][i] = nb;
        if (add) atomicAdd(&counts[0], add);
        if (over) atomicAdd(&counts[1], over);
    }
}

// ---- ParticleExchange --------------------------------------------------------
// One substep of BMXParticleContainer::ParticleExchange (bmx_pc_xchng.cpp:13-257)
// with initExchange / evaluateExchange / applyIncrements
// (bmx_chem_K.H:1949-2126): over the step's neighbour list, every FUNGI
// segment i sums, for each listed FUNGI neighbour j that i and j both hold in
// their bond tables, -d / vol_i with d = (c_i - c_j) * area * mt * dt
// (area = pi (r_i^2 + r_j^2) / 2), d clamped so that neither side loses more
// than its concentration over its bond count, and adds the sum to its
// concentrations.  The reference's write to j's increment goes to a by-value
// neighbour copy and is lost; the result reads only concentrations from
// before the substep, so the kernel writes a separate output.  Same
// arithmetic, in the same order, as the reference (FP64, no contraction).
__global__ void k_exchange(const DevState S, const DevParams P, int a, const double *vol, const double *conc,
                           double *out, double dt, double mtA, double mtB, double mtC)
{
    const int n = S.n;
    const double pi = 3.14159265358979323846;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double a1 = conc[i], b1 = conc[(size_t)n + i], c1 = conc[(size_t)2 * n + i];
        double inc[3] = {0.0, 0.0, 0.0};
        if (S.ctype[i] == kFungi) {
            const DevGeom &G = geom_of(S, i);
            int bx, by;
            col_to_bxy(G, S.col[a][i], bx, by);
            const double xi = S.x[a][i], yi = S.y[a][i], zi = S.z[a][i];
            int tb[13];
            for (int k = 0; k < 13; ++k) tb[k] = S.tab[a][(size_t)k * n + i];
            const int iid = S.id[i], icpu = S.cpu[i];
            const double r1 = S.rad[i], v1 = vol[i];
            const double area1 = pi * r1 * r1;
            const double ni = (double)tb[0];
            visit_stencil(S, G, a, i, bx, by, S.iz[a][i], [&](int j, int, int, int, int sx, int sy) {
                if (S.ctype[j] != kFungi) return;
                if (!G.nbh_trivial) {  // BMXCheckPair: j is in i's list only within the neighbourhood
                    double d[3];
                    if (!(sep64(S, G, a, j, sx, sy, xi, yi, zi, d) <= P.nbh)) return;
                }
                if (find_in_table(tb, S.id[j], S.cpu[j]) < 0) return;
                if (find_in_plane_table(S.tab[a], n, j, iid, icpu) < 0) return;
                const double a2 = conc[j], b2 = conc[(size_t)n + j], c2 = conc[(size_t)2 * n + j];
                const double r2 = S.rad[j], v2 = vol[j];
                const double area2 = pi * r2 * r2;
                const double area = 0.5 * (area1 + area2);
                const double nj = (double)S.tab[a][j];
                double dA = (a1 - a2) * area * mtA * dt;
                double dB = (b1 - b2) * area * mtB * dt;
                double dC = (c1 - c2) * area * mtC * dt;
                if (dA / v1 > a1 / ni) dA = a1 * v1 / ni;
                if (-dA / v2 > a2 / nj) dA = -a2 * v2 / nj;
                if (dB / v1 > b1 / ni) dB = b1 * v1 / ni;
                if (-dB / v2 > b2 / nj) dB = -b2 * v2 / nj;
                if (dC / v1 > c1 / ni) dC = c1 * v1 / ni;
                if (-dC / v2 > c2 / nj) dC = -c2 * v2 / nj;
                inc[0] -= dA / v1;
                inc[1] -= dB / v1;
                inc[2] -= dC / v1;
            });
        }
        out[i] = a1 + inc[0];
        out[(size_t)n + i] = b1 + inc[1];
        out[(size_t)2 * n + i] = c1 + inc[2];
    }
}

}  // namespace

int launch_exchange(const DevState &S, const DevParams &P, int a, const double *vol, const double *conc, double *out,
                    double dt, const double *xpar, int grid, int block, cudaStream_t st)
{
    k_exchange<<<grid, block, 0, st>>>(S, P, a, vol, conc, out, dt, xpar[0], xpar[1], xpar[2]);
    return 1;
}

int launch_rod_mobility(const DevState &S, const DevParams &P, int grid, int block, cudaStream_t st)
{
    k_rod_mobility<<<grid, block, 0, st>>>(S, P);
    return 1;
}

int launch_rod_book(const DevState &S, const DevParams &P, int a, bool list, int grid, int block, cudaStream_t st)
{
    if (list)
        k_rod_book<true><<<grid, block, 0, st>>>(S, P, a);
    else
        k_rod_book<false><<<grid, block, 0, st>>>(S, P, a);
    return 1;
}

int launch_rod_pairs(const DevState &S, const DevParams &P, int a, int nsm, int n, cudaStream_t st)
{
    k_rod_pair32<<<nsm * 8, 256, 0, st>>>(S, P, a);
    k_rod_pair64<<<nsm * 4, 128, 0, st>>>(S, P, a);
    k_rod_seg32<<<(n + 127) / 128, 128, 0, st>>>(S, P, a);
    return 3;
}

int launch_rod_force(const DevState &S, const DevParams &P, int a, int precision, int grid, int block,
                      cudaStream_t st)
{
    if (precision == BMXG_FP64_FORM)
        k_rod_force<BMXG_FP64_FORM><<<grid, block, 0, st>>>(S, P, a);
    else
        k_rod_force<BMXG_FP32F_FORM><<<grid, block, 0, st>>>(S, P, a);
    return 1;
}

int launch_rod_update(const DevState &S, double dt, int a, int grid, int block, cudaStream_t st)
{
    k_rod_update<<<grid, block, 0, st>>>(S, dt, a);
    return 1;
}

int launch_init_bonds(const DevState &S, const DevParams &P, int a, double rlim, unsigned long long *counts,
                      int grid, int block, cudaStream_t st)
{
    k_init_bonds<<<grid, block, 0, st>>>(S, P, a, rlim, counts);
    return 1;
}

}  // namespace bmxg
