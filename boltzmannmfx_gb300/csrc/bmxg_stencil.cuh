// bmxg_stencil.cuh -- the neighbour traversal every kernel shares, and the
// per-slot rebin.  Translation units that include this are compiled with
// -fmad=false so that every FP64 expression rounds exactly like the host
// oracle's (FP32 code uses explicit __fmaf_rn where it wants a fused op).
#pragma once
#include "bmxg_kernels.cuh"

namespace bmxg {

// Whether the periodic image of slot j under shift (sx, sy) lies in stencil
// row (ii, jj): the image's bin is computed from its shifted FP64 position,
// as AMReX bins its ghost copies.
__device__ __forceinline__ bool image_in_row(const DevState &S, const DevGeom &G, int a, int j,
                                             int ii, int jj, int sx, int sy)
{
    if (sx) {
        double gx = S.x[a][j] + (double)sx * G.len[0];
        if (bin_of(gx, G.plo[0], G.dxi[0], 0, G.n[0] + 1) != ii) return false;
    }
    if (sy) {
        double gy = S.y[a][j] + (double)sy * G.len[1];
        if (bin_of(gy, G.plo[1], G.dxi[1], 0, G.n[1] + 1) != jj) return false;
    }
    return true;
}

// Visit slot i's neighbour candidates in the order of the reference's
// neighbour list: stencil bins x outermost, then y, then z, ascending
// original index within a bin (AMReX NeighborList over the 27 bins around
// the particle's bin, periodic images from the one-cell halo).  Each column is
// entered by binary search at its first entry of z bin izi - 1.
// f(j, dxs, dys, dzs, sx, sy): dxs/dys/dzs = neighbour bin minus own bin,
// sx/sy = image shift in units of the domain length.
template <class F>
__device__ __forceinline__ void visit_stencil(const DevState &S, const DevGeom &G, int a, int i,
                                              int bx, int by, int izi, F &&f)
{
    const int *__restrict__ perm = S.perm[a];
    const int *__restrict__ cs = S.colstart[a];
    const int *__restrict__ izs = S.iz[a];
    for (int ii = bx - 1; ii <= bx + 1; ++ii) {
        for (int jj = by - 1; jj <= by + 1; ++jj) {
            int cc, sx, sy;
            if (!stencil_row(G, ii, jj, cc, sx, sy)) continue;
            const int t1 = __ldg(&cs[cc + 1]);
            int t0 = __ldg(&cs[cc]);
            for (int hi2 = t1; t0 < hi2;) {  // first entry of z bin >= izi - 1
                const int mid = (t0 + hi2) >> 1;
                if (__ldg(&izs[__ldg(&perm[mid])]) < izi - 1) t0 = mid + 1;
                else hi2 = mid;
            }
            for (int t = t0; t < t1; ++t) {
                const int j = __ldg(&perm[t]);
                const int dzs = __ldg(&izs[j]) - izi;
                if (dzs > 1) break;  // a column is sorted by z-bin: the rest is out of reach
                if (dzs < -1) continue;
                if (j == i) continue;
                if ((sx | sy) && !image_in_row(S, G, a, j, ii, jj, sx, sy)) continue;
                f(j, ii - bx, jj - by, dzs, sx, sy);
            }
        }
    }
}

// First t in [lo, hi) with siz[t] >= v (siz ascends over the range).
__device__ __forceinline__ int first_at_least(const int *__restrict__ siz, int lo, int hi, int v)
{
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(&siz[mid]) < v) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// The same walk over the column-sorted copies (siz / srel, filled by the
// rebuild): f(t, dxs, dys, dzs, sx, sy) gets the sorted index t of each
// candidate (its slot is perm[t]).  An x-row's three columns by-1..by+1 are
// consecutive column ids, so away from the periodic faces a row is three
// back-to-back runs of one contiguous range; each run is ordered by z-bin
// and is entered by binary search at its first entry of z-bin izi - 1 (a
// column can be many bins tall), and left at the first entry above izi + 1.
// self_t = rank of the slot itself.  Order of candidates: identical to
// visit_stencil.
template <class F>
__device__ __forceinline__ void visit_sorted(const DevState &S, const DevGeom &G, int a, int self_t, int bx,
                                             int by, int izi, F &&f)
{
    const int *__restrict__ cs = S.colstart[a];
    const int *__restrict__ siz = S.siz[a];
    for (int ii = bx - 1; ii <= bx + 1; ++ii) {
        int srcx = ii, sx = 0;
        if (ii == 0) {
            if (!G.per[0]) continue;
            srcx = G.n[0];
            sx = -1;
        } else if (ii == G.n[0] + 1) {
            if (!G.per[0]) continue;
            srcx = 1;
            sx = 1;
        }
        if (sx == 0 && by >= 2 && by <= G.n[1] - 1) {
            const int c = column_of(G, srcx, by - 1);
            int lo = __ldg(&cs[c]);
            for (int dys = -1; dys <= 1; ++dys) {
                const int hi = __ldg(&cs[c + dys + 2]);
                for (int t = first_at_least(siz, lo, hi, izi - 1); t < hi; ++t) {
                    const int dzs = __ldg(&siz[t]) - izi;
                    if (dzs > 1) break;
                    if (dzs < -1 || t == self_t) continue;
                    f(t, ii - bx, dys, dzs, 0, 0);
                }
                lo = hi;
            }
        } else {
            for (int jj = by - 1; jj <= by + 1; ++jj) {
                int cc, ssx, sy;
                if (!stencil_row(G, ii, jj, cc, ssx, sy)) continue;
                const int t1 = __ldg(&cs[cc + 1]);
                for (int t = first_at_least(siz, __ldg(&cs[cc]), t1, izi - 1); t < t1; ++t) {
                    const int dzs = __ldg(&siz[t]) - izi;
                    if (dzs > 1) break;
                    if (dzs < -1 || t == self_t) continue;
                    if ((ssx | sy) && !image_in_row(S, G, a, __ldg(&S.perm[a][t]), ii, jj, ssx, sy)) continue;
                    f(t, ii - bx, jj - by, dzs, ssx, sy);
                }
            }
        }
    }
}

// Walk the stencil over the column-sorted copies when the state has them
// (SORTED), else over perm (callers that provide no sorted buffers).  f gets
// the candidate's FP32 offsets, a functor returning its slot, and the shifts.
template <bool SORTED, class F>
__device__ __forceinline__ void walk(const DevState &S, const DevGeom &G, int a, int i, int bx, int by, int izi,
                                     F &&f)
{
    if constexpr (SORTED) {
        visit_sorted(S, G, a, S.rank[a][i], bx, by, izi, [&](int t, int dxs, int dys, int dzs, int sx, int sy) {
            f(__ldg(&S.srel[a][t]), [&]() { return __ldg(&S.perm[a][t]); }, dxs, dys, dzs, sx, sy);
        });
    } else {
        visit_stencil(S, G, a, i, bx, by, izi, [&](int j, int dxs, int dys, int dzs, int sx, int sy) {
            f(__ldg(&S.rel[a][j]), [&]() { return j; }, dxs, dys, dzs, sx, sy);
        });
    }
}

// Grown-box bin (bx, by) of a slot from its column id.
__device__ __forceinline__ void col_to_bxy(const DevGeom &G, int col, int &bx, int &by)
{
    const int q = col - G.col_base;
    bx = q / G.n[1] + 1;
    by = q - (bx - 1) * G.n[1] + 1;
}

// Bin a slot at position (x, y, z): column and z bin into buffer bb, FP32
// offsets from the bin corner into buffer rb, column count; flag
// out-of-domain z, images that leave their halo cell, and non-finite positions.
// place_slot does the same for bins already known.
__device__ __forceinline__ void place_slot(const DevState &S, const DevGeom &G, int i, double x, double y,
                                           double z, double r, int bb, int rb, int bx, int by, int bz,
                                           bool count_domain, bool count_col)
{
    const int c = column_of(G, bx, by);
    S.col[bb][i] = c;
    S.iz[bb][i] = bz;
    // bin corners from the geometry's table (the same FP64 formula, evaluated
    // once on the host), the conversions and tests from the bits: FP64
    // arithmetic here is the three differences (GB300 issues FP64 at a small
    // fraction of the FP32 rate)
    auto corner = [&](int d, int bin) {
        return (bin >= 1 && bin <= G.ncorner[d]) ? G.corner[d][bin - 1] : G.plo[d] + (double)(bin - 1) * G.dx[d];
    };
    const double cx = corner(0, bx), cy = corner(1, by), cz = corner(2, bz);
    S.rel[rb][i] = make_float4(d2f_rn(x - cx), d2f_rn(y - cy), d2f_rn(z - cz), d2f_rn(r));
    if (count_col) atomicAdd(&S.colcnt[c], 1);
    if (count_domain) {
        // inside for certain from the FP32 values (truncated z within 2^-21 of the
        // magnitudes), else the FP64 test
        const float zf = d2f_trunc(z);
        const float m = 4.8e-7f * (fabsf(zf) + fabsf(G.plof[2]) + fabsf(G.phif[2]));
        const bool sure = G.phif[2] > G.plof[2] && zf - m > G.plof[2] && zf + m < G.phif[2];
        if (!sure && !(z >= G.plo[2] && z < G.phi[2])) atomicAdd(&S.cnt->out_of_domain, 1ULL);
    }
    if (!finite_bits(x) || !finite_bits(y) || !finite_bits(z)) atomicAdd(&S.cnt->nonfinite, 1ULL);
    if (G.per[0] && (bx == 1 || bx == G.n[0])) {
        const int sx = (bx == 1) ? 1 : -1;
        const int gb = bin_of(x + (double)sx * G.len[0], G.plo[0], G.dxi[0], 0, G.n[0] + 1);
        if (gb != (sx > 0 ? G.n[0] + 1 : 0)) atomicAdd(&S.cnt->edge_ghost, 1ULL);
    }
    if (G.per[1] && (by == 1 || by == G.n[1])) {
        const int sy = (by == 1) ? 1 : -1;
        const int gb = bin_of(y + (double)sy * G.len[1], G.plo[1], G.dxi[1], 0, G.n[1] + 1);
        if (gb != (sy > 0 ? G.n[1] + 1 : 0)) atomicAdd(&S.cnt->edge_ghost, 1ULL);
    }
}

__device__ __forceinline__ void rebin_slot_into(const DevState &S, const DevGeom &G, int i, double x, double y,
                                                double z, double r, int bb, int rb, bool count_domain = true,
                                                bool count_col = true)
{
    const int bx = bin_of_fast(x, G.plo[0], G.dxi[0], G.plof[0], G.dxif[0], 1, G.n[0]);
    const int by = bin_of_fast(y, G.plo[1], G.dxi[1], G.plof[1], G.dxif[1], 1, G.n[1]);
    const int bz = bin_of_fast(z, G.plo[2], G.dxi[2], G.plof[2], G.dxif[2], 1, G.n[2]);
    place_slot(S, G, i, x, y, z, r, bb, rb, bx, by, bz, count_domain, count_col);
}

// Bin a slot into buffer b (bins and offsets).
__device__ __forceinline__ void rebin_slot(const DevState &S, const DevGeom &G, int i, double x, double y,
                                           double z, double r, int b)
{
    rebin_slot_into(S, G, i, x, y, z, r, b, b);
}

// Growth-surface cubic law of one site at height z
// (bmx_cell_interaction_K.H:1019-1030, :1099-1121).
__device__ __forceinline__ double wall_law(double z, double rS, const DevParams &P)
{
    const double dz = z - P.z_wall;
    const double rA = rS + P.z_bw;
    double v;
    if (dz > 0.0 && dz < rA) v = -P.z_k * (dz - rA) * (dz - rA) * (dz - rS);
    else if (dz <= 0.0) v = P.z_k * rA * rA * rS;
    else v = 0.0;
    v -= P.z_g * P.z_k * rA * rA * rS;
    return v;
}

// Exact float -> double conversion with integer operations (GB300's FP64
// pipe is the scarce resource here), on the two 32-bit words: for a normal
// float the high word is the sign, then exponent and mantissa shifted down by
// three with the exponent rebased by 1023 - 127, and the low word the last
// three mantissa bits.  Subnormal floats flush to a signed zero; infinities
// and NaNs keep their payload.
__device__ __forceinline__ double f2d_int(float f)
{
    const unsigned u = __float_as_uint(f);
    const unsigned sgn = u & 0x80000000u, a = u & 0x7fffffffu;
    unsigned hi = sgn | ((a >> 3) + 0x38000000u);
    unsigned lo = u << 29;
    if (a < 0x00800000u) {
        hi = sgn;
        lo = 0u;
    } else if (a >= 0x7f800000u) {
        hi = sgn | 0x7ff00000u | ((a & 0x7fffffu) >> 3);
    }
    return __hiloint2double((int)hi, (int)lo);
}

// growth-surface cubic law in FP32 (bmx_cell_interaction_K.H:1019-1030)
__device__ __forceinline__ float wall_law32(float dz, float rS, float zk, float zbw, float zg)
{
    const float rA = rS + zbw;
    float v;
    if (dz > 0.0f && dz < rA) v = -zk * (dz - rA) * (dz - rA) * (dz - rS);
    else if (dz <= 0.0f) v = zk * rA * rA * rS;
    else v = 0.0f;
    return v - zg * zk * rA * rA * rS;
}

__device__ __forceinline__ const DevGeom &geom_of(const DevState &S, int i)
{
    return S.geoms[colony_of(S.cbase, S.ncol, i)];
}

}  // namespace bmxg
