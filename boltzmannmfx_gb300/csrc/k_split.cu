// k_split.cu -- cell division (split_particles) on particles in the reference's
// AoS layout: YEAST cells (setNewCell) and FUNGI segments (tip extension,
// side branching, isolated halving: setNewSegment; two-way tip split:
// setNewSegments).
//
// BMXParticleContainer::split_particles (src/des/bmx_split_particles.cpp:16-166)
// runs after the DEM step: a flag pass (checkSplit, src/chemistry/bmx_chem_K.H:
// 23-69), an exclusive scan of the new-particle counts that gives each division
// the slots of its daughters past the end of the tile, a read of the total on
// the host, and a fill pass (copyChildParameters, setNewCell, setNewSegment,
// setNewSegments; bmx_chem_K.H:357-1011, 2129-2494).
//
// Random draws follow one sequence, the calls to amrex::Random of a serial run
// in their order: first checkSplit's (one for each FUNGI tip at the radius
// limit and each segment behind a tip, in array order), then the divisions'
// (in array order: 2 for a YEAST cell, 2 for a tip extension, 3 for a side
// branch, 4 for a two-way split, none for an isolated segment).  With no draw
// array a SplitMix64 counter generator keyed by (seed, id, cpu, j) supplies
// draw j of a cell: j = 0 its checkSplit draw, j = 1.. its division's.
//
// Device passes:
//   k_split_checks  per 256-particle block, the number of checkSplit draws
//                   (calls with a draw sequence only);
//   k_split_decide  each particle's decision (new particles 0..2, division
//                   draws 0..4) packed in one byte, block sums of both and of
//                   the divisions;
//   k_split_scan    exclusive scans of the block sums (one 1024-thread block
//                   per array);
//   k_split_index   the list of divisions with their daughter and draw
//                   offsets (block-local scans on the block offsets), grouped
//                   by kind of division;
//   k_split_divide  one thread per division: the warp copies its mothers'
//                   copied blocks into the daughters in coalesced rows, then
//                   each lane runs its division.
// The decision pass reads two to four words of each 448-byte record (as many
// 128-byte lines); a division reads and writes about one record per particle
// it touches.
#include <climits>
#include <cstdint>
#include <cstring>
#include <mutex>

#include <cuda_runtime.h>

#include "../../include/bmxg.h"

namespace bmxg {
namespace {

// realIdx (src/chemistry/bmx_chem.H:38-69)
enum { R_radius = 0, R_c_length = 1, R_theta = 2, R_phi = 3, R_area = 4, R_vol = 5, R_dadt = 21,
       R_dvdt = 22, R_bond_scale = 24, R_first = 25 };
// intIdx (src/chemistry/bmx_chem.H:77-118)
enum { I_cell_type = 5, I_n_bnds = 6, I_seg1_id1 = 7, I_seg2_id1 = 8, I_seg3_id1 = 9, I_seg4_id1 = 10,
       I_seg1_id2 = 11, I_seg2_id2 = 12, I_seg3_id2 = 13, I_seg4_id2 = 14, I_site1 = 15, I_site2 = 16,
       I_site3 = 17, I_site4 = 18, I_position = 19, I_fuse_flag = 20, I_split_flag = 21, I_new_flag = 22,
       I_fuse_id = 23, I_fuse_cpu = 24, I_fuse_tip = 25, I_dltd_site1 = 26, I_fix_site = 32, I_id = 33,
       I_cpu = 34, I_first = 35 };

constexpr int kBlock = 256;
constexpr int kScanThreads = 1024;
constexpr double kPi = 3.14159265358979323846;  // M_PI

struct SplitArgs {
    unsigned char *par;   // record 0 of the tile
    unsigned char *kid;   // record of new particle 0 (particles + n records, or a staging copy)
    long long n;
    long long stride;     // bytes per record
    int rdata, ids, idata;  // byte offsets of rdata[], (id, cpu), idata[] in a record
    int nreals, nints;    // copied block: reals [0, nreals), ints [0, nints)
    double max_vol, overlap, max_len, max_rad, brnch_prob, split_prob, split_len;
    int use_draws;        // 1: the draw sequence below; 0: the counter generator
    const double *draws;
    unsigned long long seed;
    long long next_id;
    int my_proc;
    long long *cnt_a;     // [nb + 1] checkSplit draws per block, then their exclusive scan
    long long *cnt_n;     // [nb + 1] new particles
    long long *cnt_d;     // [nb + 1] division draws
    long long *cnt_k;     // [nb + 1] divisions
    unsigned char *dec;   // [n] new particles | division draws << 2 | kind << 5
    int *kinds;           // [16]: divisions of each kind, then the fill counters of their regions
};

// kinds of division; the division list is grouped by kind so that a warp of
// k_split_divide runs one kind's code (the list order does not change the
// result: every entry carries its own daughter and draw offsets)
enum { kCell = 0, kTip = 1, kBranch = 2, kTwo = 3, kHalve = 4, kKinds = 5 };

struct Division {  // one entry of the division list
    int i;         // the mother
    int kid;       // first daughter, counted from new particle 0
    int draw;      // first division draw, counted in the whole sequence
    int n_new;
};

__device__ __forceinline__ double *rec_r(const SplitArgs &a, unsigned char *rec) { return (double *)(rec + a.rdata); }
__device__ __forceinline__ int *rec_i(const SplitArgs &a, unsigned char *rec) { return (int *)(rec + a.idata); }
__device__ __forceinline__ int *rec_id(const SplitArgs &a, unsigned char *rec) { return (int *)(rec + a.ids); }

// SplitMix64 (Steele, Lea and Flood, "Fast splittable pseudorandom number
// generators", OOPSLA 2014) on the counter (cpu, id, j): draw j of the cell
// with that identity, as a double in [0, 1) with 53 random bits.
__host__ __device__ __forceinline__ double split_uniform(unsigned long long seed, int id, int cpu, int j)
{
    const unsigned long long key = ((unsigned long long)(unsigned)cpu << 32) | (unsigned long long)(unsigned)id;
    unsigned long long z = seed + 0x9E3779B97F4A7C15ull * (key * 2ull + (unsigned long long)j + 1ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * 0x1.0p-53;
}

// checkSplit draws one value for a FUNGI tip at the radius limit and for a
// segment behind a tip (bmx_chem_K.H:36-66)
__device__ __forceinline__ int needs_check_draw(const SplitArgs &a, unsigned char *rec)
{
    const int *q = rec_i(a, rec);
    if (q[I_cell_type] != BMXG_FUNGI) return 0;
    const int pos = q[I_position];
    if (pos == BMXG_SITE_TIP) return rec_r(a, rec)[R_radius] >= a.max_rad ? 1 : 0;
    return (pos == BMXG_SITE_SECOND_1 || pos == BMXG_SITE_SECOND_2) ? 1 : 0;
}

// checkSplit's decision (bmx_chem_K.H:23-69) given its draw x, and the number
// of draws the division then takes (setNewCell 2; setNewSegment: isolated 0,
// tip 2, side branch 3; setNewSegments 4), packed as n_new | draws << 2 |
// kind << 5
__device__ __forceinline__ int decide(const SplitArgs &a, unsigned char *rec, double x)
{
    const int *q = rec_i(a, rec);
    const double *r = rec_r(a, rec);
    const int ct = q[I_cell_type];
    const double vol = r[R_vol];  // issued with cell_type: another line of the record
    if (ct == BMXG_YEAST) return vol > a.max_vol ? (1 | (2 << 2) | (kCell << 5)) : 0;
    if (ct != BMXG_FUNGI) return 0;
    const int pos = q[I_position], nb = q[I_n_bnds];
    if (pos == BMXG_SITE_TIP) {
        if (!(r[R_radius] >= a.max_rad) || !(r[R_c_length] >= a.max_len)) return 0;
        if (x > a.split_prob || nb == 0) return nb == 0 ? (1 | (kHalve << 5)) : (1 | (2 << 2) | (kTip << 5));
        return 2 | (4 << 2) | (kTwo << 5);
    }
    if (pos == BMXG_SITE_SECOND_1 || pos == BMXG_SITE_SECOND_2)
        return (x < a.brnch_prob) ? (nb == 0 ? (1 | (kHalve << 5)) : (1 | (3 << 2) | (kBranch << 5))) : 0;
    return 0;
}

// block-wide exclusive sum of v (blockDim.x == kBlock); *total gets the sum
__device__ __forceinline__ int block_excl(int v, int *ws, int *total)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int s = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, s, d);
        if (lane >= d) s += t;
    }
    if (lane == 31) ws[w] = s;
    __syncthreads();
    int off = 0, all = 0;
#pragma unroll
    for (int j = 0; j < kBlock / 32; ++j) {
        off += (j < w) ? ws[j] : 0;
        all += ws[j];
    }
    __syncthreads();
    *total = all;
    return off + s - v;
}

__global__ void __launch_bounds__(kBlock) k_split_checks(SplitArgs a)
{
    const long long i = (long long)blockIdx.x * kBlock + threadIdx.x;
    const int c = i < a.n ? needs_check_draw(a, a.par + i * a.stride) : 0;
    const int cnt = __syncthreads_count(c);
    if (threadIdx.x == 0) a.cnt_a[blockIdx.x] = cnt;
}

__global__ void __launch_bounds__(kBlock) k_split_decide(SplitArgs a)
{
    __shared__ int ws[kBlock / 32];
    __shared__ int sk[kKinds];
    if (threadIdx.x < kKinds) sk[threadIdx.x] = 0;
    __syncthreads();  // the counters are zero before any warp adds to them
    const long long i = (long long)blockIdx.x * kBlock + threadIdx.x;
    unsigned char *rec = a.par + (i < a.n ? i : 0) * a.stride;
    const int c = i < a.n ? needs_check_draw(a, rec) : 0;
    double x = 0.0;
    if (a.use_draws) {
        int tot;
        const int off = block_excl(c, ws, &tot);
        if (c) x = a.draws[a.cnt_a[blockIdx.x] + off];
    } else if (c) {
        const int *id = rec_id(a, rec);
        x = split_uniform(a.seed, id[0], id[1], 0);
    }
    const int d = i < a.n ? decide(a, rec, x) : 0;
    if (i < a.n) a.dec[i] = (unsigned char)d;
    // divisions of each kind: per warp into the block's counters, then one
    // global atomic per kind and block (the block_excl barriers below order them)
    const int kind = (d & 3) ? (d >> 5) : -1;
    const unsigned same = __match_any_sync(0xffffffffu, kind);
    if (kind >= 0 && (threadIdx.x & 31) == __ffs(same) - 1) atomicAdd(&sk[kind], __popc(same));
    int tn, td, tk;
    block_excl(d & 3, ws, &tn);
    block_excl((d >> 2) & 7, ws, &td);
    block_excl((d & 3) ? 1 : 0, ws, &tk);
    if (threadIdx.x == 0) {
        a.cnt_n[blockIdx.x] = tn;
        a.cnt_d[blockIdx.x] = td;
        a.cnt_k[blockIdx.x] = tk;
    }
    if (threadIdx.x < kKinds && sk[threadIdx.x]) atomicAdd(&a.kinds[threadIdx.x], sk[threadIdx.x]);
}

// exclusive scan of c[0, nb) in place, total in c[nb]; block b scans array b
__global__ void __launch_bounds__(kScanThreads) k_split_scan(long long *c0, long long *c1, long long *c2, int nb)
{
    __shared__ long long s[kScanThreads];
    long long *c = blockIdx.x == 0 ? c0 : (blockIdx.x == 1 ? c1 : c2);
    const int t = threadIdx.x;
    const int per = (nb + kScanThreads - 1) / kScanThreads;
    const long long lo = (long long)t * per;
    const long long hi = lo + per < nb ? lo + per : nb;
    long long sum = 0;
    for (long long j = lo; j < hi; ++j) sum += c[j];
    s[t] = sum;
    __syncthreads();
    for (int d = 1; d < kScanThreads; d <<= 1) {
        const long long v = t >= d ? s[t - d] : 0;
        __syncthreads();
        s[t] += v;
        __syncthreads();
    }
    long long run = s[t] - sum;
    for (long long j = lo; j < hi; ++j) {
        const long long v = c[j];
        c[j] = run;
        run += v;
    }
    if (t == kScanThreads - 1) c[nb] = s[t];
}

// the divisions with their daughters' and draws' offsets (from the array-order
// scans), grouped by kind: the kinds' regions follow each other in kind order,
// and within a region the entries land in arrival order
__global__ void __launch_bounds__(kBlock) k_split_index(SplitArgs a, Division *list, long long checks)
{
    __shared__ int ws[kBlock / 32];
    __shared__ int sk[kKinds], sb[kKinds];
    if (threadIdx.x < kKinds) sk[threadIdx.x] = 0;
    const long long i = (long long)blockIdx.x * kBlock + threadIdx.x;
    const int d = i < a.n ? a.dec[i] : 0;
    int t;
    const int on = block_excl(d & 3, ws, &t);
    const int od = block_excl((d >> 2) & 7, ws, &t);
    // a slot in the kind's region: the warp's share of the block's, the
    // block's share of the region's (one global atomic per kind and block)
    const int kind = (d & 3) ? (d >> 5) : -1;
    const unsigned same = __match_any_sync(0xffffffffu, kind);
    const int lane = threadIdx.x & 31, lead = __ffs(same) - 1;
    int slot = 0;
    if (kind >= 0 && lane == lead) slot = atomicAdd(&sk[kind], __popc(same));
    slot = __shfl_sync(0xffffffffu, slot, lead) + __popc(same & ((1u << lane) - 1u));
    __syncthreads();
    if (threadIdx.x < kKinds) sb[threadIdx.x] = sk[threadIdx.x] ? atomicAdd(&a.kinds[kKinds + threadIdx.x], sk[threadIdx.x]) : 0;
    __syncthreads();
    if (kind < 0) return;
    int base = sb[kind];
    for (int k = 0; k < kind; ++k) base += a.kinds[k];
    Division e;
    e.i = (int)i;
    e.kid = (int)(a.cnt_n[blockIdx.x] + on);
    e.draw = (int)(checks + a.cnt_d[blockIdx.x] + od);
    e.n_new = d & 3;
    list[base + slot] = e;
}

// draw j of a division: from the sequence, or the counter generator (j + 1)
struct Draws {
    const double *u;
    unsigned long long seed;
    int id, cpu;
    __device__ double operator()(int j) const { return u ? u[j] : split_uniform(seed, id, cpu, j + 1); }
};

// setNewCell (bmx_chem_K.H:383-440) after the copy of the mother's block.
// Here and below the expressions keep the reference's order and grouping; the
// library is built without FMA contraction.
__device__ void divide_cell(const SplitArgs &a, unsigned char *mrec, unsigned char *drec, const Draws &u)
{
    double *mp = (double *)mrec, *dp = (double *)drec;
    double *mr = rec_r(a, mrec), *dr = rec_r(a, drec);
    int *di = rec_i(a, drec);
    const double x = mp[0], y = mp[1], z = mp[2];
    double radius = mr[R_radius];
    double theta = 2.0 * u(0) - 1.0;
    theta = acos(theta);
    const double phi = 2.0 * kPi * u(1);
    double st, ct, sp, cp;
    sincos(theta, &st, &ct);
    sincos(phi, &sp, &cp);
    const double nx = st * cp, ny = st * sp, nz = ct;
    const double scale = 1.0 - a.overlap;
    dp[0] = x + scale * 0.5 * nx * radius;
    dp[1] = y + scale * 0.5 * ny * radius;
    dp[2] = z + scale * 0.5 * nz * radius;
    mp[0] = x - scale * 0.5 * nx * radius;
    mp[1] = y - scale * 0.5 * ny * radius;
    mp[2] = z - scale * 0.5 * nz * radius;
    const double volume = mr[R_vol] / 2.0;
    radius = pow((3.0 * volume / (4.0 * kPi)), 1.0 / 3.0);
    const double area = 4.0 * kPi * radius * radius;
    const double dadt = 2.0 * mr[R_dvdt] / radius;
    mr[R_vol] = volume;
    dr[R_vol] = volume;
    mr[R_area] = area;
    dr[R_area] = area;
    mr[R_dadt] = dadt;
    dr[R_dadt] = dadt;
    mr[R_radius] = radius;
    dr[R_radius] = radius;
    dr[R_bond_scale] = 1.0;
    di[I_fuse_tip] = 0;
    for (int j = 6; j < 9; ++j) mr[R_first + j] = 0.5 * mr[R_first + j];
    for (int j = 6; j < 9; ++j) dr[R_first + j] = 0.5 * dr[R_first + j];
}

// the polar angles of a unit vector as the reference recovers them: theta =
// acos(z), phi = acos(x / sin theta) mirrored for y < 0, phi = 0 on the axis
__device__ __forceinline__ void angles_of(double x, double y, double z, double &th, double &st, double &ph)
{
    th = acos(z);
    st = sin(th);
    ph = 0.0;
    if (st != 0.0) {
        ph = acos(x / st);
        if (y < 0.0) ph = 2.0 * kPi - ph;
    }
}

// the rotation taking the x axis to the direction (sin t, cos t = gct, phi)
// applied to a direction drawn within 0.1 rad of the x axis
// (bmx_chem_K.H:612-643): g = R (cos rt, sin rt sin rp, sin rt cos rp),
// rt = 0.1 u0, rp = 2 pi u1
__device__ __forceinline__ void draw_around(double gst, double gct, double gphi, double u0, double u1,
                                            double &gnx, double &gny, double &gnz)
{
    double gsp, gcp;
    sincos(gphi, &gsp, &gcp);
    const double r00 = gcp * gst, r01 = -gsp, r02 = -gcp * gct;
    const double r10 = gsp * gst, r11 = gcp, r12 = -gsp * gct;
    const double r20 = gct, r21 = 0.0, r22 = gst;
    const double rtheta = 0.1 * u0;
    const double rphi = 2.0 * kPi * u1;
    double rst, rct, rsp, rcp;
    sincos(rtheta, &rst, &rct);
    sincos(rphi, &rsp, &rcp);
    const double rx = rct, ry = rst * rsp, rz = rst * rcp;
    gnx = r00 * rx + r01 * ry + r02 * rz;
    gny = r10 * rx + r11 * ry + r12 * rz;
    gnz = r20 * rx + r21 * ry + r22 * rz;
}

// a new tip's flags and deleted-bond slots as the reference resets them
__device__ __forceinline__ void reset_tip(int *q, bool dltd, bool new_flag)
{
    q[I_position] = BMXG_SITE_TIP;
    q[I_fuse_flag] = 0;
    q[I_split_flag] = 0;
    if (new_flag) q[I_new_flag] = 0;
    q[I_fuse_id] = -1;
    q[I_fuse_cpu] = -1;
    if (dltd)
        for (int j = 0; j < 6; ++j) q[I_dltd_site1 + j] = -1;
}

__device__ __forceinline__ void seg_vol_area(double *r)
{
    const double clen = r[R_c_length], rad = r[R_radius];
    r[R_vol] = kPi * rad * rad * clen;
    r[R_area] = 2.0 * kPi * rad * clen + 2.0 * kPi * rad * rad;
}

// setNewSegment (bmx_chem_K.H:457-1011) after the copy of the mother's block:
// an isolated segment halves; a tip at the length limit shortens to split_len
// and a new tip grows from its free end; a segment behind a tip grows a side
// branch of length 5e-4 from the end the tip hangs on.  The chemical gradient
// is zero in the reference (:468-473), so the growth direction is the
// segment's own (tip) or one at +-45 degrees in the xy plane (side branch).
__device__ void divide_segment(const SplitArgs &a, unsigned char *mrec, unsigned char *drec, const Draws &u,
                               int id, int cpu)
{
    double *mp = (double *)mrec, *dp = (double *)drec;
    double *mr = rec_r(a, mrec), *dr = rec_r(a, drec);
    int *mi = rec_i(a, mrec), *di = rec_i(a, drec);
    const int nbnd = mi[I_n_bnds];
    const int position = mi[I_position];
    if (nbnd == 0) {
        const double x_orig = mp[0], y_orig = mp[1], z_orig = mp[2];
        const double c_length = mr[R_c_length];
        double st, ct, sp, cp;
        sincos(mr[R_theta], &st, &ct);
        sincos(mr[R_phi], &sp, &cp);
        const double nx = st * cp, ny = st * sp, nz = ct;
        mp[0] = x_orig + 0.25 * c_length * nx;
        mp[1] = y_orig + 0.25 * c_length * ny;
        mp[2] = z_orig + 0.25 * c_length * nz;
        dp[0] = x_orig - 0.25 * c_length * nx;
        dp[1] = y_orig - 0.25 * c_length * ny;
        dp[2] = z_orig - 0.25 * c_length * nz;
        mr[R_c_length] = 0.5 * c_length;
        dr[R_c_length] = 0.5 * c_length;
        mi[I_n_bnds] = 1;
        mi[I_seg1_id1] = id;
        mi[I_seg1_id2] = cpu;
        mi[I_site1] = 1;
        reset_tip(mi, true, true);
        di[I_n_bnds] = 1;
        di[I_seg1_id1] = mi[I_id];
        di[I_seg1_id2] = mi[I_cpu];
        di[I_site1] = 2;
        reset_tip(di, true, true);
        di[I_fix_site] = 0;
        for (int j = 6; j < 9; ++j) mr[R_first + j] = 0.5 * mr[R_first + j];
        for (int j = 6; j < 9; ++j) dr[R_first + j] = 0.5 * dr[R_first + j];
    } else if (position == BMXG_SITE_TIP) {
        const int bsite = mi[I_site1];
        double st, ct, sp, cp;
        sincos(mr[R_theta], &st, &ct);
        sincos(mr[R_phi], &sp, &cp);
        const double nx = st * cp, ny = st * sp, nz = ct;
        // zero gradient: the growth direction is the segment's own (gn = 1)
        const double gx = nx / 1.0, gy = ny / 1.0, gz = nz / 1.0;
        double gtheta, gst, gphi;
        angles_of(gx, gy, gz, gtheta, gst, gphi);
        double gnx, gny, gnz;
        draw_around(gst, gz, gphi, u(0), u(1), gnx, gny, gnz);
        const double x = mp[0], y = mp[1], z = mp[2];
        const double c_length = mr[R_c_length];
        const double split_len = a.split_len;
        const double seg_len = c_length - split_len;
        double ax, ay, az, ex, ey, ez;  // the new tip's far end, and the shared end
        if (bsite == 1) {
            const double x1 = x - 0.5 * c_length * nx, y1 = y - 0.5 * c_length * ny, z1 = z - 0.5 * c_length * nz;
            ex = x1 + split_len * nx;
            ey = y1 + split_len * ny;
            ez = z1 + split_len * nz;
            mp[0] = 0.5 * (x1 + ex);
            mp[1] = 0.5 * (y1 + ey);
            mp[2] = 0.5 * (z1 + ez);
            mr[R_c_length] = split_len;
            if (nbnd == 1) mi[I_site2] = 2;
            else mi[I_site3] = 2;
            mi[I_position] = BMXG_SITE_SECOND_2;
            ax = ex + gnx * seg_len;
            ay = ey + gny * seg_len;
            az = ez + gnz * seg_len;
        } else {
            const double x2 = x + 0.5 * c_length * nx, y2 = y + 0.5 * c_length * ny, z2 = z + 0.5 * c_length * nz;
            ex = x2 - split_len * nx;
            ey = y2 - split_len * ny;
            ez = z2 - split_len * nz;
            mp[0] = 0.5 * (ex + x2);
            mp[1] = 0.5 * (ey + y2);
            mp[2] = 0.5 * (ez + z2);
            mr[R_c_length] = split_len;
            if (nbnd == 1) mi[I_site2] = 1;
            else mi[I_site3] = 1;
            mi[I_position] = BMXG_SITE_SECOND_1;
            ax = ex - gnx * seg_len;
            ay = ey - gny * seg_len;
            az = ez - gnz * seg_len;
        }
        dp[0] = 0.5 * (ex + ax);
        dp[1] = 0.5 * (ey + ay);
        dp[2] = 0.5 * (ez + az);
        dr[R_c_length] = seg_len;
        double nth, nst, nph;
        angles_of(gnx, gny, gnz, nth, nst, nph);
        dr[R_theta] = nth;
        dr[R_phi] = nph;
        di[I_site1] = bsite == 1 ? 1 : 2;
        reset_tip(di, bsite == 1, true);
        di[I_fix_site] = 0;
        if (nbnd == 1) {
            mi[I_n_bnds] = 2;
            mi[I_seg2_id1] = id;
            mi[I_seg2_id2] = cpu;
        } else {
            mi[I_n_bnds] = 3;
            mi[I_seg3_id1] = id;
            mi[I_seg3_id2] = cpu;
        }
        di[I_n_bnds] = 1;
        di[I_seg1_id1] = mi[I_id];
        di[I_seg1_id2] = mi[I_cpu];
        for (int j = 6; j < 9; ++j) dr[R_first + j] = 0.0;
    } else if (position == BMXG_SITE_SECOND_1 || position == BMXG_SITE_SECOND_2) {
        const double theta = mr[R_theta], phi = mr[R_phi];
        double st, ct, sp, cp;
        sincos(theta, &st, &ct);
        sincos(phi, &sp, &cp);
        const double nx = st * cp, ny = st * sp, nz = ct;
        // zero gradient: +-45 degrees from phi in the xy plane
        const double da = u(0) > 0.5 ? 0.25 * kPi : -0.25 * kPi;
        const double tphi = phi + da;
        double stp, ctp;
        sincos(tphi, &stp, &ctp);
        const double gx = ctp / 1.0, gy = stp / 1.0, gz = 0.0 / 1.0;
        double gtheta, gst, gphi;
        angles_of(gx, gy, gz, gtheta, gst, gphi);
        double gnx, gny, gnz;
        draw_around(gst, gz, gphi, u(1), u(2), gnx, gny, gnz);
        double gntheta, gnst, gnphi;
        angles_of(gnx, gny, gnz, gntheta, gnst, gnphi);
        const double x = mp[0], y = mp[1], z = mp[2];
        const double c_length = mr[R_c_length];
        const double seg_len = 0.0005;
        if (position == BMXG_SITE_SECOND_1) {
            if (nbnd == 2) mi[I_site3] = 1;
            else if (nbnd == 3) mi[I_site4] = 1;
            const double x1 = x - 0.5 * c_length * nx, y1 = y - 0.5 * c_length * ny, z1 = z - 0.5 * c_length * nz;
            const double ax = x1 - gnx * seg_len, ay = y1 - gny * seg_len, az = z1 - gnz * seg_len;
            dp[0] = 0.5 * (x1 + ax);
            dp[1] = 0.5 * (y1 + ay);
            dp[2] = 0.5 * (z1 + az);
            di[I_site1] = 2;
            di[I_site2] = 2;
        } else {
            if (nbnd == 2) mi[I_site3] = 2;
            else if (nbnd == 3) mi[I_site4] = 2;
            const double x2 = x + 0.5 * c_length * nx, y2 = y + 0.5 * c_length * ny, z2 = z + 0.5 * c_length * nz;
            const double ax = x2 + gnx * seg_len, ay = y2 + gny * seg_len, az = z2 + gnz * seg_len;
            dp[0] = 0.5 * (x2 + ax);
            dp[1] = 0.5 * (y2 + ay);
            dp[2] = 0.5 * (z2 + az);
            di[I_site1] = 1;
            di[I_site2] = 1;
        }
        double radius = mr[R_radius];
        const double old_vol = c_length * radius * radius * kPi;
        dr[R_theta] = gntheta;
        dr[R_phi] = gnphi;
        // the daughter still holds the mother's length here (:939)
        radius = old_vol / (kPi * (c_length + dr[R_c_length]));
        radius = sqrt(radius);
        mr[R_radius] = radius;
        dr[R_radius] = radius;
        dr[R_c_length] = seg_len;
        if (nbnd == 2) {
            mi[I_n_bnds] = 3;
            mi[I_seg3_id1] = id;
            mi[I_seg3_id2] = cpu;
        } else {
            mi[I_n_bnds] = 4;
            mi[I_seg4_id1] = id;
            mi[I_seg4_id2] = cpu;
        }
        di[I_n_bnds] = 2;
        di[I_seg1_id1] = mi[I_id];
        di[I_seg1_id2] = mi[I_cpu];
        if (nbnd == 2) {
            di[I_seg2_id1] = mi[I_seg2_id1];
            di[I_seg2_id2] = mi[I_seg2_id2];
        } else {
            di[I_seg2_id1] = mi[I_seg3_id1];
            di[I_seg2_id2] = mi[I_seg3_id2];
        }
        reset_tip(di, true, true);
        di[I_fix_site] = 0;
        mi[I_position] = BMXG_SITE_INTERIOR;
        for (int j = 6; j < 9; ++j) dr[R_first + j] = 0.0;
    }
    di[I_id] = id;
    di[I_cpu] = cpu;
    seg_vol_area(mr);
    seg_vol_area(dr);
    dr[R_bond_scale] = 1.0;
    di[I_fuse_tip] = 0;
}

// setNewSegments (bmx_chem_K.H:2129-2494) after the copies of the mother's
// block: a tip splits in two at +-45 degrees in the xy plane; the mother keeps
// split_len of its bonded end and both daughters take half the rest.
__device__ void divide_tip_in_two(const SplitArgs &a, unsigned char *mrec, unsigned char *d1rec,
                                  unsigned char *d2rec, const Draws &u, int id1, int cpu1, int id2, int cpu2)
{
    double *mp = (double *)mrec, *p1 = (double *)d1rec, *p2 = (double *)d2rec;
    double *mr = rec_r(a, mrec), *r1 = rec_r(a, d1rec), *r2 = rec_r(a, d2rec);
    int *mi = rec_i(a, mrec), *i1 = rec_i(a, d1rec), *i2 = rec_i(a, d2rec);
    const double phi = mr[R_phi];
    double st, ct, sp, cp;
    sincos(mr[R_theta], &st, &ct);
    sincos(phi, &sp, &cp);
    const double nx = st * cp, ny = st * sp, nz = ct;
    const double da = 0.25 * kPi;
    const double tphi1 = phi + da, tphi2 = phi - da;
    double gy1, gx1, gy2, gx2;
    sincos(tphi1, &gy1, &gx1);
    sincos(tphi2, &gy2, &gx2);
    const double gz1 = 0.0, gz2 = 0.0;
    double th, gst1, gphi1, gst2, gphi2;
    angles_of(gx1, gy1, gz1, th, gst1, gphi1);
    angles_of(gx2, gy2, gz2, th, gst2, gphi2);
    double gnx1, gny1, gnz1, gnx2, gny2, gnz2;
    draw_around(gst1, gz1, gphi1, u(0), u(1), gnx1, gny1, gnz1);
    draw_around(gst2, gz2, gphi2, u(2), u(3), gnx2, gny2, gnz2);
    double gntheta1, gnst1, gnphi1, gntheta2, gnst2, gnphi2;
    angles_of(gnx1, gny1, gnz1, gntheta1, gnst1, gnphi1);
    angles_of(gnx2, gny2, gnz2, gntheta2, gnst2, gnphi2);
    const double x = mp[0], y = mp[1], z = mp[2];
    const double c_length = mr[R_c_length];
    const double seg_len = 0.5 * (c_length - a.split_len);
    const double new_len = c_length - 2.0 * seg_len;
    const int site = mi[I_site1] == 1 ? 1 : 2;  // the daughters' site at the shared end
    const int msite = site == 1 ? 2 : 1;         // the mother's end they grow from
    if (site == 1) {
        const double x1 = x - 0.5 * c_length * nx, y1 = y - 0.5 * c_length * ny, z1 = z - 0.5 * c_length * nz;
        const double newx = x1 + new_len * nx, newy = y1 + new_len * ny, newz = z1 + new_len * nz;
        mp[0] = 0.5 * (x1 + newx);
        mp[1] = 0.5 * (y1 + newy);
        mp[2] = 0.5 * (z1 + newz);
        double ax = newx + gnx1 * seg_len, ay = newy + gny1 * seg_len, az = newz + gnz1 * seg_len;
        p1[0] = 0.5 * (newx + ax);
        p1[1] = 0.5 * (newy + ay);
        p1[2] = 0.5 * (newz + az);
        ax = newx + gnx2 * seg_len;
        ay = newy + gny2 * seg_len;
        az = newz + gnz2 * seg_len;
        p2[0] = 0.5 * (newx + ax);
        p2[1] = 0.5 * (newy + ay);
        p2[2] = 0.5 * (newz + az);
    } else {
        const double x2 = x + 0.5 * c_length * nx, y2 = y + 0.5 * c_length * ny, z2 = z + 0.5 * c_length * nz;
        const double newx = x2 - new_len * nx, newy = y2 - new_len * ny, newz = z2 - new_len * nz;
        mp[0] = 0.5 * (x2 + newx);
        mp[1] = 0.5 * (y2 + newy);
        mp[2] = 0.5 * (z2 + newz);
        double ax = newx - gnx1 * seg_len, ay = newy - gny1 * seg_len, az = newz - gnz1 * seg_len;
        p1[0] = 0.5 * (newx + ax);
        p1[1] = 0.5 * (newy + ay);
        p1[2] = 0.5 * (newz + az);
        ax = newx - gnx2 * seg_len;
        ay = newy - gny2 * seg_len;
        az = newz - gnz2 * seg_len;
        p2[0] = 0.5 * (newx + ax);
        p2[1] = 0.5 * (newy + ay);
        p2[2] = 0.5 * (newz + az);
    }
    // each daughter bonds to the mother and to its sister at the shared end
    i1[I_site1] = site;
    i1[I_seg1_id1] = mi[I_id];
    i1[I_seg1_id2] = mi[I_cpu];
    i1[I_site2] = site;
    i1[I_seg2_id1] = id2;
    i1[I_seg2_id2] = cpu2;
    i1[I_n_bnds] = 2;
    i2[I_site1] = site;
    i2[I_seg1_id1] = mi[I_id];
    i2[I_seg1_id2] = mi[I_cpu];
    i2[I_site2] = site;
    i2[I_seg2_id1] = id1;
    i2[I_seg2_id2] = cpu1;
    i2[I_n_bnds] = 2;
    if (mi[I_n_bnds] == 1) {
        mi[I_site2] = msite;
        mi[I_seg2_id1] = id1;
        mi[I_seg2_id2] = cpu1;
        mi[I_site3] = msite;
        mi[I_seg3_id1] = id2;
        mi[I_seg3_id2] = cpu2;
        mi[I_n_bnds] = 3;
    } else {
        mi[I_site3] = msite;
        mi[I_seg3_id1] = id1;
        mi[I_seg3_id2] = cpu1;
        mi[I_site4] = msite;
        mi[I_seg4_id1] = id2;
        mi[I_seg4_id2] = cpu2;
        mi[I_n_bnds] = 4;
    }
    mr[R_c_length] = new_len;
    r1[R_c_length] = seg_len;
    r2[R_c_length] = seg_len;
    r1[R_theta] = gntheta1;
    r1[R_phi] = gnphi1;
    r2[R_theta] = gntheta2;
    r2[R_phi] = gnphi2;
    reset_tip(i1, true, false);
    i1[I_fix_site] = 0;
    reset_tip(i2, true, false);
    i2[I_fix_site] = 0;
    mi[I_position] = BMXG_SITE_INTERIOR;
    i1[I_id] = id1;
    i1[I_cpu] = cpu1;
    i2[I_id] = id2;
    i2[I_cpu] = cpu2;
    seg_vol_area(mr);
    seg_vol_area(r1);
    r1[R_bond_scale] = 1.0;
    i1[I_fuse_tip] = 0;
    seg_vol_area(r2);
    r2[R_bond_scale] = 1.0;
    i2[I_fuse_tip] = 0;
}

// One thread per division over the compacted list, so that the FP64
// transcendental functions of a division run with full warps (a few percent of
// the cells divide in a step; one thread per cell would leave most lanes
// idle).  First the warp copies the copied block (copyChildParameters) of its
// mothers into their daughters: the (daughter, word) pairs are spread over the
// lanes, kCopyUnroll loads in flight per lane before their stores.  Small
// blocks (kDivBlock): a step divides a few thousand cells, which must still
// cover every SM.
constexpr int kDivBlock = 64;
constexpr int kCopyUnroll = 8;

template <typename T>
__device__ __forceinline__ void copy_block(const SplitArgs &a, const int *src, const int *dst, int nd, int lane,
                                           int nwords, int off)
{
    const int total = nd * nwords;
    for (int t0 = lane; t0 < total; t0 += 32 * kCopyUnroll) {
        T v[kCopyUnroll];
#pragma unroll
        for (int u = 0; u < kCopyUnroll; ++u) {
            const int t = t0 + 32 * u;
            if (t < total) {
                const int j = t / nwords, w = t - j * nwords;
                v[u] = ((const T *)(a.par + (long long)src[j] * a.stride + off))[w];
            }
        }
#pragma unroll
        for (int u = 0; u < kCopyUnroll; ++u) {
            const int t = t0 + 32 * u;
            if (t < total) {
                const int j = t / nwords, w = t - j * nwords;
                ((T *)(a.kid + (long long)dst[j] * a.stride + off))[w] = v[u];
            }
        }
    }
}

__global__ void __launch_bounds__(kDivBlock) k_split_divide(SplitArgs a, const Division *list, long long total)
{
    __shared__ int src[kDivBlock * 2], dst[kDivBlock * 2];
    const long long k0 = (long long)blockIdx.x * kDivBlock + (threadIdx.x & ~31);
    if (k0 >= total) return;
    const int lane = threadIdx.x & 31;
    const long long k = k0 + lane;
    Division e;
    e.i = 0;
    e.kid = 0;
    e.draw = 0;
    e.n_new = 0;
    if (k < total) e = list[k];
    // the warp's daughters: every division's first, then the second ones
    const unsigned two = __ballot_sync(0xffffffffu, e.n_new == 2);
    const int nk = total - k0 < 32 ? (int)(total - k0) : 32;
    int *ws = src + 2 * (threadIdx.x & ~31), *wd = dst + 2 * (threadIdx.x & ~31);
    if (lane < nk) {
        ws[lane] = e.i;
        wd[lane] = e.kid;
        if (e.n_new == 2) {
            const int r = __popc(two & ((1u << lane) - 1u));
            ws[nk + r] = e.i;
            wd[nk + r] = e.kid + 1;
        }
    }
    __syncwarp();
    const int nd = nk + __popc(two);
    copy_block<double>(a, ws, wd, nd, lane, a.nreals, a.rdata);
    copy_block<int>(a, ws, wd, nd, lane, a.nints, a.idata);
    __syncwarp();
    if (k >= total) return;
    unsigned char *mrec = a.par + (long long)e.i * a.stride;
    unsigned char *d1 = a.kid + (long long)e.kid * a.stride;
    const int *mid = rec_id(a, mrec);
    Draws u;
    u.u = a.use_draws ? a.draws + e.draw : nullptr;
    u.seed = a.seed;
    u.id = mid[0];
    u.cpu = mid[1];
    const int id1 = (int)(a.next_id + e.kid);
    int *s1 = rec_id(a, d1);
    if (e.n_new == 2) {
        unsigned char *d2 = d1 + a.stride;
        divide_tip_in_two(a, mrec, d1, d2, u, id1, a.my_proc, id1 + 1, a.my_proc);
        int *s2 = rec_id(a, d2);
        s2[0] = id1 + 1;
        s2[1] = a.my_proc;
    } else {
        if (rec_i(a, mrec)[I_cell_type] == BMXG_YEAST) divide_cell(a, mrec, d1, u);
        else divide_segment(a, mrec, d1, u, id1, a.my_proc);
        rec_i(a, d1)[I_id] = id1;
        rec_i(a, d1)[I_cpu] = a.my_proc;
    }
    s1[0] = id1;
    s1[1] = a.my_proc;
}

// Per-device scratch kept across calls (the block sums, the decisions, the
// division list, and a pinned block for the host's read of the totals); it
// grows to the largest call and is held until the process exits.  One call at
// a time per device uses it (the mutex is held for the whole call).
struct DevScratch {
    std::mutex mu;
    unsigned char *dev = nullptr;
    size_t dev_bytes = 0;
    long long *host = nullptr;
};
constexpr int kMaxDevices = 64;
DevScratch g_scratch[kMaxDevices];

// stream-ordered staging buffers of host-memory calls, released on return
struct Staging {
    cudaStream_t st;
    void *p[3] = {nullptr, nullptr, nullptr};
    int used = 0;
    explicit Staging(cudaStream_t s) : st(s) {}
    void *get(size_t bytes)
    {
        if (used == 3) return nullptr;
        void *q = nullptr;
        if (cudaMallocAsync(&q, bytes, st) != cudaSuccess) return nullptr;
        p[used++] = q;
        return q;
    }
    ~Staging()
    {
        for (int j = 0; j < used; ++j) cudaFreeAsync(p[j], st);
        cudaStreamSynchronize(st);
    }
};

size_t align256(size_t b) { return (b + 255) / 256 * 256; }

}  // namespace
}  // namespace bmxg

using namespace bmxg;

#define SPLIT_CK(call)                                  \
    do {                                                \
        if ((call) != cudaSuccess) return BMXG_ERR_CUDA; \
    } while (0)

extern "C" int bmxg_split_cells_aos(const bmxg_split_params *sp, void *particles, int64_t n, int64_t cap,
                                    int32_t nreal, int32_t nint, const double *draws, int64_t ndraws,
                                    uint64_t seed, int64_t next_id, int32_t my_proc, int32_t where,
                                    int64_t *num_split, void *stream)
{
    if (!sp || !num_split || n < 0 || cap < n) return BMXG_ERR_ARG;
    *num_split = 0;
    if (where != BMXG_HOST && where != BMXG_DEVICE) return BMXG_ERR_ARG;
    // the species increments first_data + 6..8 are written whatever num_reals is
    if (nreal < R_first + 9 || nint < I_first) return BMXG_ERR_ARG;
    if (sp->num_reals < 0 || sp->num_ints < 0 || R_first + sp->num_reals > nreal ||
        I_first + sp->num_ints > nint)
        return BMXG_ERR_ARG;
    // the reference's indices are ints: up to two daughters per particle
    if (n > INT_MAX / 3 || cap > INT_MAX || ndraws < 0 || ndraws > INT_MAX) return BMXG_ERR_ARG;
    if (n == 0) return BMXG_OK;
    if (!particles || ((uintptr_t)particles & 7u)) return BMXG_ERR_ARG;
    if (draws && ((uintptr_t)draws & 7u)) return BMXG_ERR_ARG;
    int dev = 0;
    SPLIT_CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return BMXG_ERR_UNSUPPORTED;

    SplitArgs a;
    std::memset(&a, 0, sizeof(a));
    a.rdata = 3 * (int)sizeof(double);
    a.ids = a.rdata + nreal * (int)sizeof(double);
    a.idata = a.ids + 2 * (int)sizeof(int);
    a.stride = ((long long)a.idata + (long long)nint * (long long)sizeof(int) + 7) / 8 * 8;
    a.n = n;
    a.nreals = R_first + sp->num_reals;
    a.nints = I_first + sp->num_ints;
    a.max_vol = sp->max_vol;
    a.overlap = sp->overlap;
    a.max_len = sp->max_len;
    a.max_rad = sp->max_rad;
    a.brnch_prob = sp->brnch_prob;
    a.split_prob = sp->split_prob;
    a.split_len = sp->split_len;
    a.use_draws = draws ? 1 : 0;
    a.seed = seed;
    a.next_id = next_id;
    a.my_proc = my_proc;

    cudaStream_t st = static_cast<cudaStream_t>(stream);
    DevScratch &S = g_scratch[dev];
    std::lock_guard<std::mutex> lock(S.mu);
    const long long nb = (n + kBlock - 1) / kBlock;
    // four block-sum arrays [nb + 1], the kind counters, the decisions [n], the list [n]
    const size_t sums = align256(sizeof(long long) * (size_t)(nb + 1));
    const size_t off_kinds = 4 * sums;
    const size_t off_dec = off_kinds + 256;
    const size_t off_list = align256(off_dec + (size_t)n);
    const size_t need = off_list + sizeof(Division) * (size_t)n;
    if (!S.host) SPLIT_CK(cudaMallocHost((void **)&S.host, 4 * sizeof(long long)));
    if (S.dev_bytes < need) {
        SPLIT_CK(cudaStreamSynchronize(st));
        if (S.dev) SPLIT_CK(cudaFree(S.dev));
        S.dev = nullptr;
        S.dev_bytes = 0;
        if (cudaMalloc((void **)&S.dev, need) != cudaSuccess) return BMXG_ERR_OOM;
        S.dev_bytes = need;
    }
    a.cnt_a = (long long *)S.dev;
    a.cnt_n = (long long *)(S.dev + sums);
    a.cnt_d = (long long *)(S.dev + 2 * sums);
    a.cnt_k = (long long *)(S.dev + 3 * sums);
    a.dec = S.dev + off_dec;
    a.kinds = (int *)(S.dev + off_kinds);
    Division *list = (Division *)(S.dev + off_list);

    Staging stage(st);
    const size_t rec_bytes = (size_t)n * (size_t)a.stride;
    if (where == BMXG_DEVICE) {
        a.par = static_cast<unsigned char *>(particles);
    } else {
        a.par = (unsigned char *)stage.get(rec_bytes);
        if (!a.par) return BMXG_ERR_OOM;
        SPLIT_CK(cudaMemcpyAsync(a.par, particles, rec_bytes, cudaMemcpyHostToDevice, st));
    }
    // with a draw sequence, checkSplit's draws come first: count them (a host
    // sequence is staged whole: its used length is known only after the
    // decisions)
    long long checks = 0;
    if (draws) {
        if (where == BMXG_DEVICE) {
            a.draws = draws;
        } else if (ndraws > 0) {
            double *d = (double *)stage.get(sizeof(double) * (size_t)ndraws);
            if (!d) return BMXG_ERR_OOM;
            SPLIT_CK(cudaMemcpyAsync(d, draws, sizeof(double) * (size_t)ndraws, cudaMemcpyHostToDevice, st));
            a.draws = d;
        }
        k_split_checks<<<(unsigned)nb, kBlock, 0, st>>>(a);
        k_split_scan<<<1, kScanThreads, 0, st>>>(a.cnt_a, a.cnt_a, a.cnt_a, (int)nb);
        SPLIT_CK(cudaGetLastError());
        SPLIT_CK(cudaMemcpyAsync(S.host, a.cnt_a + nb, sizeof(long long), cudaMemcpyDeviceToHost, st));
        SPLIT_CK(cudaStreamSynchronize(st));
        checks = S.host[0];
        if (ndraws < checks) return BMXG_ERR_ARG;  // too short for checkSplit's own draws
    }
    SPLIT_CK(cudaMemsetAsync(a.kinds, 0, 16 * sizeof(int), st));
    k_split_decide<<<(unsigned)nb, kBlock, 0, st>>>(a);
    k_split_scan<<<3, kScanThreads, 0, st>>>(a.cnt_n, a.cnt_d, a.cnt_k, (int)nb);
    SPLIT_CK(cudaGetLastError());
    SPLIT_CK(cudaMemcpyAsync(S.host + 1, a.cnt_n + nb, sizeof(long long), cudaMemcpyDeviceToHost, st));
    SPLIT_CK(cudaMemcpyAsync(S.host + 2, a.cnt_d + nb, sizeof(long long), cudaMemcpyDeviceToHost, st));
    SPLIT_CK(cudaMemcpyAsync(S.host + 3, a.cnt_k + nb, sizeof(long long), cudaMemcpyDeviceToHost, st));
    SPLIT_CK(cudaStreamSynchronize(st));
    const long long total = S.host[1], ndraw = S.host[2], ndiv = S.host[3];
    *num_split = total;
    if (total == 0) return BMXG_OK;
    if (n + total > cap) return BMXG_ERR_CAPACITY;
    if (draws && ndraws < checks + ndraw) return BMXG_ERR_ARG;

    unsigned char *host_kids = static_cast<unsigned char *>(particles) + rec_bytes;
    const size_t kid_bytes = (size_t)total * (size_t)a.stride;
    if (where == BMXG_DEVICE) {
        a.kid = a.par + rec_bytes;
    } else {
        // the new records start from what the caller's buffer holds, so the
        // fields a division leaves unset come back unchanged
        a.kid = (unsigned char *)stage.get(kid_bytes);
        if (!a.kid) return BMXG_ERR_OOM;
        SPLIT_CK(cudaMemcpyAsync(a.kid, host_kids, kid_bytes, cudaMemcpyHostToDevice, st));
    }
    k_split_index<<<(unsigned)nb, kBlock, 0, st>>>(a, list, checks);
    k_split_divide<<<(unsigned)((ndiv + kDivBlock - 1) / kDivBlock), kDivBlock, 0, st>>>(a, list, ndiv);
    SPLIT_CK(cudaGetLastError());
    if (where == BMXG_HOST) {
        SPLIT_CK(cudaMemcpyAsync(particles, a.par, rec_bytes, cudaMemcpyDeviceToHost, st));
        SPLIT_CK(cudaMemcpyAsync(host_kids, a.kid, kid_bytes, cudaMemcpyDeviceToHost, st));
    }
    SPLIT_CK(cudaStreamSynchronize(st));
    return BMXG_OK;
}
