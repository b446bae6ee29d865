// bmxg_dev.cuh -- device-side data layout and helpers of the DEM step.
//
// Layout in HBM (all structure-of-arrays, one entry per particle "slot").
// Slots are the particles sorted once, at bmxg_set_state, by the canonical
// neighbour-list key (colony, column, z-bin, original index); that order is
// kept for the lifetime of the state, so neighbours that the stencil visits
// sit close together in memory.  What changes every step is
//   - positions x/y/z (FP64, ping-pong A/B),
//   - the packed bin of each slot (column id + z bin, ping-pong),
//   - the per-column start offsets and the column-sorted slot list `perm`
//     (ping-pong), rebuilt by a counting sort every step exactly as the
//     reference rebuilds its neighbour list every step
//     (src/des/bmx_pc_interaction.cpp:97-103).
// A "column" is the (x-bin, y-bin) pair of one colony; a column holds its
// particles sorted by (z-bin, original index), so the three z-bins of a
// stencil row are one contiguous run -- the order in which AMReX's
// NeighborList walks its 27 bins (x outermost, z innermost, ascending index
// within a bin).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace bmxg {

constexpr double kPi = 3.14159265358979323846;  // M_PI as the reference uses it
constexpr double kSmall = 1.0e-15;              // small_number, bmx_pc_interaction.cpp:157
constexpr int BMXG_FP64_FORM = 0;               // BMXG_FP64 of bmxg.h
constexpr int BMXG_FP32F_FORM = 1;              // BMXG_FP32F of bmxg.h
constexpr int kYeast = 0, kFungi = 1;           // cellType (src/chemistry/bmx_chem.H:120-126)
constexpr int kTip = 0, kSecond1 = 1, kSecond2 = 2, kInterior = 3;  // siteLocation (bmx_chem.H:128-136)
constexpr int kWallTable = 66;                  // z-bins with a precomputed wall height (grown box)
constexpr int kCornerTable = 128;               // bins per axis with a precomputed FP64 corner
constexpr int kResyncEvery = 8;                 // FP32F: exact FP64 re-binning of every slot each 8th step

// Geometry of one colony (an AMReX level geometry) plus its place in the
// global column / slot numbering.
struct DevGeom {
    double plo[3], phi[3], len[3], dx[3], dxi[3];
    float dxf[3];
    float plof[3], dxif[3];  // plo and dxi rounded to FP32 (bin_of_fast; 0: not set, FP64 binning)
    float phif[3];           // phi rounded to FP32 (0 with plof: not set)
    int ncorner[3];          // entries of corner (0: not set)
    double corner[3][kCornerTable];  // plo + (b - 1) dx of bin b, rounded as the device formula
    int n[3];
    int per[3];
    int col_base;       // first global column of this colony
    int cell_base;      // first global 3D cell (column-major, z fastest) of this colony
    int slot_base;      // first slot of this colony
    int slot_end;       // one past the last slot
    int nbh_trivial;    // 1: BMXCheckPair's r^2 <= neighborhood holds for every stencil pair
    float invny;        // 1 / n[1], for the column -> (x-bin, y-bin) split
    int nwz;            // entries of wz (0: table not built, z too fine)
    // height of each z-bin's lower face above the growth surface,
    // (plo_z + (bz-1) dz) - z_wall, as an unevaluated float pair (hi + lo):
    // the FP32 precision form evaluates the wall law from it and the particle's
    // FP32 offset without FP64 arithmetic
    float2 wz[kWallTable];
};

// 64-bit fixed-point positions of the FP32F list path (one record per colony):
// per axis X = (x - o) / u with u = span / 2^64 and X in [0, 2^64).  A
// periodic axis spans the domain (o = plo, span = len: the unsigned wrap of X
// is the periodic wrap, and the int32 difference of two high words is the
// minimum-image offset); a closed axis spans 4 lengths from one length below
// plo, so the domain is the high word in [2^30, 2^31).
struct alignas(16) FxGeom {
    float uh[3];                // span / 2^32: the unit of the high word (pair offsets)
    unsigned zw;                // high word of the growth surface z_wall (z axis)
    float c[3];                 // 2^64 / span as an FP32 pair c + cl (an increment in units)
    float pad0;
    float cl[3];
    float pad1;
    int n[3];                   // bins per axis (the list build's cells)
    int per[3];
    int pad[2];
    double o[3], u[3];          // origin and unit (FP64: conversions at the path's ends)
    double plo[3], phi[3];      // the domain (clamp of converted periodic positions)
    // integer conversions: span = ms 2^es exactly (ms the 53-bit significand),
    // 2^64 / span = mc 2^ec with mc in [2^63, 2^64) (truncated)
    unsigned long long ms[3], mc[3];
    int es[3], ec[3];
    int ozero[3];               // the origin is 0 (no FP64 addition)
    int pad2;
};

// Counters a step accumulates on the device.
struct DevCounters {
    unsigned long long out_of_domain;
    unsigned long long edge_ghost;
    unsigned long long nonfinite;
    unsigned long long bad_index;  // counting-sort slots outside 0..n-1 (skipped; an internal error, sticky)
    unsigned long long pairs;
    unsigned long long bond_repairs;
    unsigned long long moved;
    unsigned long long range;      // list path: a z left the fixed-point range (sticky)
};

// Force parameters, fpar[0..8] (src/chemistry/bmx_cell_interaction.cpp:84-93).
struct DevParams {
    double bw, k, z_wall, z_bw, z_k, z_g, k_bond, bond_cutoff, visc, nbh;
    // bw, k, z_k, z_bw, z_g rounded to FP32 on the host for the FP32F list
    // kernels (a conversion per thread is an FP64-pipe instruction)
    float bw32, k32, z_k32, z_bw32, z_g32;
};

// Bin index along one axis in the coordinates of the box grown by one cell:
// (int)((x - plo)*dxi - lo) with lo = -1, as AMReX's NeighborList bins.
// Explicit round-to-nearest intrinsics keep it free of FMA contraction so
// the bins are bit-identical to the host oracle's.  Clamped to [lo_c, hi_c].
__device__ __forceinline__ int bin_of(double x, double plo, double dxi, int lo_c, int hi_c)
{
    double v = __dadd_rn(__dmul_rn(__dsub_rn(x, plo), dxi), 1.0);
    if (!(v > (double)lo_c)) return lo_c;
    if (v >= (double)hi_c + 1.0) return hi_c;
    return (int)v;
}

// Truncation of a double to FP32 from its bits (no FP64 instruction):
// within |x| 2^-23 of x where |x| is in the normal FP32 range, 0 for a zero,
// NaN otherwise (callers then take their FP64 path).
__device__ __forceinline__ float d2f_trunc(double x)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    if ((b << 1) == 0ull) return 0.0f;
    const unsigned hi = (unsigned)(b >> 32);
    const int e = (int)((hi >> 20) & 0x7ffu) - 1023;
    if (e < -126 || e > 127) return __int_as_float(0x7fc00000);
    return __uint_as_float((hi & 0x80000000u) | ((unsigned)(e + 127) << 23) | (unsigned)((b >> 29) & 0x7fffffu));
}

// bin_of, exactly, mostly without FP64 arithmetic (GB300 issues FP64 at a
// small fraction of the FP32 rate): v = (x - plo) dxi + 1 in FP32 from the
// truncated x and the FP32 plo, dxi is within
// 2^-20 ((|x| + |plo|) dxi + |v|) of the real value, which bounds the
// truncation, the FP32 roundings and the FP64 formula's own roundings with
// margin; when that interval holds no integer, the floor is the FP64
// formula's, and the clamps of bin_of reduce to clamping the floor.
// Otherwise (and for geometries without the FP32 values) bin_of itself.
__device__ __forceinline__ int bin_of_fast(double x, double plo, double dxi, float plof, float dxif, int lo_c,
                                           int hi_c)
{
    const float xf = d2f_trunc(x);
    const float v = __fmaf_rn(__fsub_rn(xf, plof), dxif, 1.0f);
    const float e = __fmul_rn(__fmaf_rn(fabsf(xf) + fabsf(plof), fabsf(dxif), fabsf(v)), 9.5367431640625e-07f);
    const float f0 = floorf(__fsub_rn(v, e)), f1 = floorf(__fadd_rn(v, e));
    if (f0 == f1 && dxif > 0.0f && fabsf(f0) < 1.0e7f) return min(max((int)f0, lo_c), hi_c);
    return bin_of(x, plo, dxi, lo_c, hi_c);
}

// Round-to-nearest double -> float from the bits (no FP64 instruction) where
// the result is a normal float, the FP32 conversion otherwise; equal to it.
__device__ __forceinline__ float d2f_rn(double x)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned e = (unsigned)(b >> 52) & 0x7ffu;
    if (e < 897u || e > 1150u) return (float)x;
    const unsigned m23 = (unsigned)(b >> 29) & 0x7fffffu;
    const unsigned rem = (unsigned)b & 0x1fffffffu;
    const unsigned up = (rem > 0x10000000u || (rem == 0x10000000u && (m23 & 1u))) ? 1u : 0u;
    return __uint_as_float((((unsigned)(b >> 32)) & 0x80000000u) + ((e - 896u) << 23) + m23 + up);
}

// x is neither infinite nor NaN (bit test)
__device__ __forceinline__ bool finite_bits(double x)
{
    return ((((unsigned long long)__double_as_longlong(x)) >> 52) & 0x7ffull) != 0x7ffull;
}

// AMReX enforcePeriodic restated: shift by the domain length until inside,
// then clamp against round-off.  Loops are bounded (a finite x leaves the
// loop after |x|/len + 1 iterations; a non-finite x is caught by the caller).
__device__ __forceinline__ double wrap1(double x, double lo, double hi, double len)
{
    if (x > hi) {
        for (int it = 0; x > hi && it < 64; ++it) x = __dsub_rn(x, len);
        if (x < lo) x = lo;
    } else if (x < lo) {
        for (int it = 0; x < lo && it < 64; ++it) x = __dadd_rn(x, len);
        if (x > hi) x = hi;
    }
    return x;
}

// Colony of a slot: binary search over the compact colony offsets (one
// kilobyte for 256 colonies, resident in L1, where the geometry records are
// ~0.7 KB apart).
__device__ __forceinline__ int colony_of(const int *cbase, int ncol, int slot)
{
    if (ncol == 1) return 0;
    int lo = 0, hi = ncol - 1;
    while (lo < hi) {  // last colony whose first slot <= slot
        int mid = (lo + hi + 1) >> 1;
        if (__ldg(&cbase[mid]) <= slot) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Global column id of grown-box bin coordinates (bx, by) in 1..n.
__device__ __forceinline__ int column_of(const DevGeom &g, int bx, int by)
{
    return g.col_base + (bx - 1) * g.n[1] + (by - 1);
}

// One stencil row (ii, jj) of a particle in grown bin (bx, by): the source
// column whose particles (or their periodic images) fill that row, and the
// image shift.  Returns false when the row lies outside a non-periodic face.
__device__ __forceinline__ bool stencil_row(const DevGeom &g, int ii, int jj, int &col, int &sx, int &sy)
{
    int srcx = ii, srcy = jj;
    sx = 0;
    sy = 0;
    if (ii == 0) { if (!g.per[0]) return false; srcx = g.n[0]; sx = -1; }
    else if (ii == g.n[0] + 1) { if (!g.per[0]) return false; srcx = 1; sx = 1; }
    if (jj == 0) { if (!g.per[1]) return false; srcy = g.n[1]; sy = -1; }
    else if (jj == g.n[1] + 1) { if (!g.per[1]) return false; srcy = 1; sy = 1; }
    col = column_of(g, srcx, srcy);
    return true;
}

// Pack (z-bin, original index) into the 64-bit key that orders a column.
__device__ __forceinline__ unsigned long long col_key(int iz, int orig)
{
    return ((unsigned long long)(unsigned)iz << 32) | (unsigned)orig;
}

}  // namespace bmxg
