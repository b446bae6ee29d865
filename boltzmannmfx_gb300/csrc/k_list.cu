// k_list.cu -- FP32F sphere step over a neighbour list with a skin.
//
// The force acts only on pairs closer than rA = r_i + r_j + bw
// (maxInteractionDistance and the gate r^2 <= (r_lm - 1e-15)^2,
// bmx_cell_interaction_K.H:23-40, bmx_pc_interaction.cpp:212).  When the
// largest rA is at most the smallest bin width, any pair that close sits in
// neighbouring bins, so the reference's stencil list holds it whatever the
// binning is.  The list built here holds every pair closer than rA + skin
// at build time; while no pair's separation has changed by the skin since,
// it still holds every pair closer than rA.  The pair set of a step is
// therefore the reference's; only the FP32 rounding of the pair math (the
// precision form) differs from it.
//
// State: while the list path runs, positions live in 64-bit fixed point
// (FxGeom: one unit is span / 2^64, 7e-21 cm on a 0.128 cm box, finer than
// the FP64 ulp anywhere above 2^-9 cm) as a 16-byte record per slot (the high
// 32 bits of x, y, z and the FP32 radius) and three 32-bit low words.  A
// step reads and writes those 28 bytes, reads the list and writes the FP32
// velocity; a neighbour's offset is the int32 difference of two high words
// (exact; the minimum periodic image by the unsigned wrap), converted once to
// FP32 -- one 16-byte gather per neighbour, the same line its owner reads.
// The FP32 increment, scaled to units to 2^-44 of itself, is added exactly:
// no rounding accumulates in the positions, and no FP64 instruction runs
// (GB300 issues FP64 at 1/64 of the FP32 rate).  The FP64 positions are converted from the
// fixed point whenever anything reads them (launch_list_to_fp64), and to it
// when the list path starts.
// k_list_decide bounds the separation change of every pair from the spread
// of each step's increments and asks for a build when the bound reaches the
// skin (or after max_age steps); inside a CUDA graph the build kernels sit
// in a conditional node that the decision switches, so a step without a
// build launches two kernels.
//
// Build: bins from the high words (integer arithmetic, consistent with the
// positions), a counting sort into the x-y columns, the in-column order by z
// bin and caller index (deterministic lists and FP32 summation order), the 3D
// cells' offsets from the sorted z bins, and the stencil walk that keeps
// every candidate within rA + skin on exact fixed-point differences.
//
// Roofline: the step kernel streams 28 bytes of position state in and out,
// the list in and the FP32 velocity out; the neighbour records it gathers
// are L2-resident.  HBM bound, no contraction.
#include <algorithm>

#include "bmxg_stencil.cuh"

namespace bmxg {

namespace {

// Order-preserving unsigned key of a float (and back): atomicMin / atomicMax
// on the keys order the floats.
__device__ __forceinline__ unsigned fkey(float f)
{
    const unsigned b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

__device__ __forceinline__ float funkey(unsigned k)
{
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

constexpr unsigned kKeyPosInf = 0xff800000u;  // fkey(+inf)
constexpr unsigned kKeyNegInf = 0x007fffffu;  // fkey(-inf)

// An FP32 increment f in fixed-point units, f 2^64 / span, with the constant
// as an FP32 pair c + cl (2^-48 of it): p = f c rounded, its exact error from
// an FMA, plus f cl; each part rounded to the nearest unit.  Within 2^-44 of
// the increment (and a few units: ~1e-19 cm on a 0.128 cm box), far below
// the FP64 position's own rounding; the sum into the position is exact, so
// no rounding accumulates however small the increment is against the
// position.  An increment of a quarter span or more (or a non-finite one)
// sets `big`.
__device__ __forceinline__ long long fx_inc(float f, float c, float cl, bool &big)
{
    const float p = __fmul_rn(f, c);
    if (!(fabsf(p) < 4.6116860184273879e18f)) {  // 2^62
        big = true;
        return 0ll;
    }
    const float r = __fmaf_rn(f, cl, __fmaf_rn(f, c, -p));
    // the remainder (|r| <= 2^-24 |p| + |f cl| < 2^31 below |p| = 2^54) converted
    // to a 32-bit integer: the same value, one 64-bit conversion (an FP64-pipe
    // instruction on GB300) fewer
    if (fabsf(p) < 1.8014398509481984e16f) return __float2ll_rn(p) + (long long)__float2int_rn(r);  // 2^54
    return __float2ll_rn(p) + __float2ll_rn(r);
}

__device__ __forceinline__ unsigned long long fx_join(unsigned h, unsigned l)
{
    return ((unsigned long long)h << 32) | l;
}

// The bound: for any pair, the separation change since the build is, per
// component, at most the sum over steps of the spread (largest minus
// smallest) of that step's increments; its length at most the length of
// those sums.  Unlike twice the largest displacement, it does not count a
// drift common to all slots (here: the rise of the slots below the growth
// surface).  Each step adds eps_step per component for the FP32 rounding of
// the pair offsets the gate sees.
// It also clears the per-step counters (no memset nodes in the step).
__global__ void k_list_decide(ListCtl *c, DevCounters *cnt, cudaGraphConditionalHandle h, int use_h)
{
    cnt->out_of_domain = 0ull;
    cnt->edge_ghost = 0ull;
    cnt->pairs = 0ull;
    cnt->bond_repairs = 0ull;
    cnt->moved = 0ull;
    float r2 = 0.0f;
    float rg[3];
    for (int k = 0; k < 3; ++k) {
        const unsigned lo = c->inc_min[k], hi = c->inc_max[k];
        // no slot reported (empty state): no spread
        const float spread = (hi >= lo) ? (funkey(hi) - funkey(lo)) : 0.0f;
        rg[k] = c->range[k] + spread * 1.000001f + c->eps_step;
        r2 += rg[k] * rg[k];
        c->inc_min[k] = kKeyPosInf;
        c->inc_max[k] = kKeyNegInf;
    }
    const float acc = sqrtf(r2);
    const int age = c->age + 1;
    const bool rb = c->force != 0 || !(acc <= c->skin) || age > c->max_age;
    if (rb) {
        for (int k = 0; k < 3; ++k) c->range[k] = 0.0f;
        c->acc = 0.0f;
        c->age = 0;
        c->force = 0;
        c->builds += 1;
        c->overflow = 0ull;
    } else {
        for (int k = 0; k < 3; ++k) c->range[k] = rg[k];
        c->acc = acc;
        c->age = age;
    }
    c->rebuild = rb ? 1 : 0;
    if (use_h) cudaGraphSetConditional(h, rb ? 1u : 0u);
}

// Colony of index i for a kernel whose blocks take consecutive indices, one
// per thread: one binary search per block (the colonies of a block's range
// are few), then each thread steps forward.  Slot order and the list's sorted
// order hold the colonies in the same ranges (a colony's particles stay
// together under the sort), so either index works.  Every thread of the
// block must call it (it synchronises the block).
__device__ __forceinline__ int block_colony(const DevState &S, int i)
{
    __shared__ int c0;
    if (threadIdx.x == 0) c0 = colony_of(S.cbase, S.ncol, min((int)(blockIdx.x * blockDim.x), S.n - 1));
    __syncthreads();
    int c = c0;
    while (c + 1 < S.ncol && __ldg(&S.cbase[c + 1]) <= i) ++c;
    return c;
}

// Bin of a high word: a periodic axis spans the domain (bin = h n / 2^32);
// a closed axis has the domain in [2^30, 2^31), clamped to 1..n.
__device__ __forceinline__ int fx_bin(unsigned h, int nb, int per)
{
    if (per) return (int)__umulhi(h, (unsigned)nb) + 1;
    const long long d = (long long)h - (1ll << 30);
    if (d < 0) return 1;
    const long long b = (d * nb) >> 30;
    return (b >= nb) ? nb : (int)b + 1;
}

// Bins of buffer a's fixed-point positions into the list bins (kListBins
// buffer) and the column counts.
__global__ void k_list_rebin(const DevState S, int a)
{
    if (!S.lctl->rebuild) return;
    constexpr int B = kListBins;
    if (blockIdx.x == 0 && threadIdx.x == 0) S.lctl->body_runs += 1ull;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int col = block_colony(S, i);
    if (i < S.n) {
        const DevGeom &G = S.geoms[col];
        const FxGeom &F = S.fxg[col];
        const int4 h = S.fxh[a][i];
        const int bx = fx_bin((unsigned)h.x, F.n[0], F.per[0]);
        const int by = fx_bin((unsigned)h.y, F.n[1], F.per[1]);
        const int bz = fx_bin((unsigned)h.z, F.n[2], F.per[2]);
        const int c = column_of(G, bx, by);
        S.col[B][i] = c;
        S.iz[B][i] = bz;
        atomicAdd(&S.colcnt[c], 1);
    }
}

// The order key of a slot inside its column: z bin, then caller index (the
// sorted order is column, z bin, caller index, as the 3D cells hold it).
__device__ __forceinline__ unsigned long long list_key(int bz, int orig)
{
    return ((unsigned long long)(unsigned)bz << 32) | (unsigned)orig;
}

// counting sort into the columns (arrival order from the atomics): each slot's
// key at the position it drew
__global__ void k_list_scatter(const DevState S)
{
    if (!S.lctl->rebuild) return;
    constexpr int B = kListBins;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < S.n) {
        const int c = S.col[B][i];
        const int r = atomicSub(&S.colcnt[c], 1) - 1;  // leaves colcnt at zero
        const int t = S.colstart[B][c] + r;
        if (t >= 0 && t < S.n) S.lkey[t] = list_key(S.iz[B][i], S.orig[i]);
        else atomicAdd(&S.cnt->bad_index, 1ULL);
    }
}

// deterministic order inside a column (z bin, then ascending original index:
// the slot's rank among its column's keys), and the sorted copies the build
// walks: the position record, z bin, slot, and each slot's rank
__global__ void k_list_canon(const DevState S, int a)
{
    if (!S.lctl->rebuild) return;
    constexpr int B = kListBins;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < S.n) {
        const int c = S.col[B][i];
        const int bz = S.iz[B][i];
        const int s0 = max(S.colstart[B][c], 0), s1 = min(S.colstart[B][c + 1], S.n);
        const unsigned long long me = list_key(bz, S.orig[i]);
        int rank = 0;
        for (int t = s0; t < s1; ++t) rank += (__ldg(&S.lkey[t]) < me);
        const int t = s0 + rank;
        if (t >= s1) {  // i is not among its column's members: inconsistent counts
            atomicAdd(&S.cnt->bad_index, 1ULL);
        } else {
            S.perm[B][t] = i;
            reinterpret_cast<int4 *>(S.srel[B])[t] = S.fxh[a][i];
            S.siz[B][t] = bz;
            S.rank[B][i] = t;
        }
        if ((i & 31) == 0) S.xcnt[i >> 5] = 0;  // the build adds up each group's entries
    }
}

// The 3D cells' offsets in the sorted copies from the columns' sorted z bins:
// cell (column, z) starts at the column's first position whose z bin is z or
// more.  One thread per column of the colony blockIdx.x (kCellsBlock columns
// per block, blocks strided over blockIdx.y) walks its column's members once
// and leaves the offsets of kCellsZ z bins at a time in shared memory; the
// block then writes its columns' cells, which lie together, in whole rows.
// The last entry (one past the last cell) is n.
constexpr int kCellsBlock = 128;
constexpr int kCellsZ = 32;  // one z bin per lane in the write-out

__global__ void __launch_bounds__(kCellsBlock) k_list_cells(const DevState S)
{
    if (!S.lctl->rebuild) return;
    constexpr int B = kListBins;
    constexpr int R = kCellsZ + 1;  // row pitch (no bank conflicts between the columns' rows)
    __shared__ int off[kCellsBlock * R];
    const DevGeom &G = S.geoms[blockIdx.x];
    const int nz = G.n[2];
    const int ncols = G.n[0] * G.n[1];
    for (int q0 = blockIdx.y * kCellsBlock; q0 < ncols; q0 += gridDim.y * kCellsBlock) {  // same trip count
        const int q = q0 + threadIdx.x;
        const int nq = min(kCellsBlock, ncols - q0);
        // t: the column's first position whose z bin (v; past the column's
        // end: above every bin) is not below the current z
        int t = 0, s1 = 0;
        if (q < ncols) {
            t = max(__ldg(&S.colstart[B][G.col_base + q]), 0);
            s1 = min(__ldg(&S.colstart[B][G.col_base + q + 1]), S.n);
        }
        int v = (t < s1) ? __ldg(&S.siz[B][t]) : 0x7fffffff;
        for (int zc = 0; zc < nz; zc += kCellsZ) {
            const int zl = min(kCellsZ, nz - zc);
            if (q < ncols) {
                for (int k = 0; k < zl; ++k) {
                    const int z = zc + k + 1;
                    while (v < z) {
                        ++t;
                        v = (t < s1) ? __ldg(&S.siz[B][t]) : 0x7fffffff;
                    }
                    off[threadIdx.x * R + k] = t;
                }
            }
            __syncthreads();
            // the block's cells of this z range: a warp writes one column's zl
            // cells at a time, lane k the k-th (a whole row; the columns' rows
            // lie one after another when nz <= kCellsZ)
            const int lane = threadIdx.x & 31;
            int *dst = S.cellstart + G.cell_base + (size_t)q0 * nz + zc;
            if (lane < zl)
                for (int cq = threadIdx.x >> 5; cq < nq; cq += kCellsBlock / 32)
                    dst[(size_t)cq * nz + lane] = off[cq * R + lane];
            __syncthreads();
        }
    }
    if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) S.cellstart[S.ncells_total] = S.n;
}

// Visit the slots of the 3 x 3 neighbour columns of bin (bx, by), z bins
// izi - 1 .. izi + 1 (periodic images included), as contiguous cell ranges
// of the sorted copies: f(u) for each sorted position u but the slot's own
// self_t (SKIP_SELF; otherwise f sees it too and excludes it itself).  Order:
// x rows outermost, then y, then z, ascending caller index within a cell.
template <bool SKIP_SELF = true, class F>
__device__ __forceinline__ void visit_cells(const DevState &S, const DevGeom &G, int self_t, int bx, int by, int izi,
                                            F &&f)
{
    const int *__restrict__ cs = S.cellstart;
    const int nz = G.n[2];
    const int z0 = max(izi - 1, 1), z1 = min(izi + 1, nz);
    for (int dxs = -1; dxs <= 1; ++dxs) {
        int sx = bx + dxs;
        if (sx < 1 || sx > G.n[0]) {
            if (!G.per[0]) continue;
            sx += (sx < 1) ? G.n[0] : -G.n[0];
        }
        for (int dys = -1; dys <= 1; ++dys) {
            int sy = by + dys;
            if (sy < 1 || sy > G.n[1]) {
                if (!G.per[1]) continue;
                sy += (sy < 1) ? G.n[1] : -G.n[1];
            }
            const int cb = G.cell_base + ((sx - 1) * G.n[1] + (sy - 1)) * nz;
            const int hi = __ldg(&cs[cb + z1]);
            for (int u = __ldg(&cs[cb + z0 - 1]); u < hi; ++u) {
                if (SKIP_SELF && u == self_t) continue;
                f(u);
            }
        }
    }
}

// Entries of slot i's list past the inline ones that the step takes from
// the compacted list (none for a slot whose list overflowed: it walks).
__device__ __forceinline__ int list_extra(int cnt)
{
    return (cnt > kNbrInline && cnt <= kNbrCap) ? cnt - kNbrInline : 0;
}

// List build: every slot (in sorted order, so a warp's lanes share cells)
// keeps the neighbours closer than rA + skin on the exact fixed-point
// differences of the high words (+ a slack of four units per component and
// the FP32 rounding of the test), and its list length.  The rounding margin:
// the offsets' unit factors are scaled by 1 - 1e-6 (r^2 by 1 - 2e-6), against
// at most ~4e-7 of relative FP32 rounding in r^2 and in the bound squared;
// the slot's own record passes the test (distance 0) and is dropped after it.
__global__ void __launch_bounds__(256, 6) k_list_build(const DevState S, const DevParams P)
{
    if (!S.lctl->rebuild) return;
    constexpr int B = kListBins;
    const int n = S.n;
    const float reach = P.bw32 + S.lctl->skin;
    const int4 *__restrict__ sg = reinterpret_cast<const int4 *>(S.srel[B]);
    unsigned long long over = 0;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int col = block_colony(S, t);  // the sorted order keeps the colonies' ranges
    if (t < n) {
        const int i = S.perm[B][t];
        const DevGeom &G = S.geoms[col];
        const FxGeom &F = S.fxg[col];
        int bx, by;
        col_to_bxy(G, S.col[B][i], bx, by);
        const int izi = S.siz[B][t];
        const int4 me = sg[t];
        const float ri = __int_as_float(me.w);
        const float ci = ri + (reach + 4.0f * (F.uh[0] + F.uh[1] + F.uh[2]));  // the bound less r_j
        const float ux = F.uh[0] * 0.999999f, uy = F.uh[1] * 0.999999f, uz = F.uh[2] * 0.999999f;
        int c = 0;
        int4 rec = make_int4(0, 0, 0, 0);
        visit_cells<false>(S, G, t, bx, by, izi, [&](int s) {
            const int4 q = __ldg(&sg[s]);
            const float ex = (float)(me.x - q.x) * ux;
            const float ey = (float)(me.y - q.y) * uy;
            const float ez = (float)(me.z - q.z) * uz;
            const float r2f = __fmaf_rn(ex, ex, __fmaf_rn(ey, ey, __fmul_rn(ez, ez)));
            const float lim = __int_as_float(q.w) + ci;
            if (!(r2f <= lim * lim) || s == t) return;
            const int e = __ldg(&S.perm[B][s]);
            if (c == 0) rec.y = e;
            else if (c == 1) rec.z = e;
            else if (c == 2) rec.w = e;
            else if (c < kNbrCap) S.nbr[(size_t)(c - kNbrInline) * n + i] = e;
            ++c;
        });
        rec.x = min(c, 255);
        S.lrec[i] = rec;
        if (c > kNbrCap) ++over;
        const int x = list_extra(rec.x);  // its group's count of entries past the inline ones
        if (x) atomicAdd(&S.xcnt[i >> 5], x);
    }
    if (over) atomicAdd(&S.lctl->overflow, over);
}

// Gated pairs of a step, recorded when the context asks (S.pcap): per slot,
// the count and the neighbour slots the step accumulated, in its order.
struct PairRec {
    int *cap;
    int i, k;
    __device__ __forceinline__ void add(int j)
    {
        if (cap && k < kPairCap) cap[(size_t)i * (kPairCap + 1) + 1 + k] = j;
        ++k;
    }
    __device__ __forceinline__ void done()
    {
        if (cap) cap[(size_t)i * (kPairCap + 1)] = k;
    }
};

// Compaction of the list entries past the inline ones, per group of 32
// consecutive slots (the step's warps): the groups' counts (added up by
// k_list_build into counts that k_list_canon zeroed), then (after their
// exclusive scan into xoff) each slot's entries copied from the build's
// planes to xlist[xoff[group] + the entries of the group's earlier slots].
// One slot per thread, whole warps.

__global__ void k_list_xcopy(const DevState S)
{
    if (!S.lctl->rebuild) return;
    const int n = S.n;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const int x = (i < n) ? list_extra(S.lrec[i].x & 0xff) : 0;
    int o = x;  // inclusive scan over the warp
    for (int d = 1; d < 32; d <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, o, d);
        if (lane >= d) o += v;
    }
    if (x) {
        int *dst = S.xlist + __ldg(&S.xoff[i >> 5]) + (o - x);
        for (int k = 0; k < x; ++k) dst[k] = __ldg(&S.nbr[(size_t)k * n + i]);
    }
    // the slot's place in its group's run beside the list length (bits 8-17:
    // at most 31 x 29 entries precede it)
    if (i < n) S.lrec[i].x = (S.lrec[i].x & 0xff) | ((o - x) << 8);
}

// FP32F sphere step over the list: pair offsets from the fixed-point high
// words, pair math and wall law in FP32, the increments added in 64-bit fixed
// point (the periodic wrap is the unsigned wrap; the domain test of the
// closed z axis compares the high word).
// Each block takes a contiguous chunk of slots (a multiple of 32), so a
// thread's colony is found by one binary search and then by stepping forward
// from the last one.  The list metadata and the first entries come in one
// 16-byte record; the rest (a slot's list is mostly 0 to 3 long, rarely up to
// a dozen) from the compacted list, where a warp's entries lie together: a
// few sectors per warp, not one per entry as a plane per list position would
// cost.
template <bool CAP, bool PERSIST>
__global__ void __launch_bounds__(256, 6) k_list_step(const DevState S, const DevParams P, float dtf, int a, int chunk)
{
    constexpr int B = kListBins;
    const int b = a ^ 1;
    const int n = S.n;
    const float bwf = P.bw32, kf = P.k32;
    const float zkf = P.z_k32, zbwf = P.z_bw32, zgf = P.z_g32;
    const int4 *__restrict__ ga = S.fxh[a];
    const unsigned *__restrict__ la = S.fxl[a];
    // smallest and largest increment per component (order-preserving keys),
    // per warp in shared memory: reduced over the warp after each pass, so
    // that no register holds them through the list walk
    __shared__ unsigned wmin[32][3], wmax[32][3];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (lane < 3) {
        wmin[w][lane] = kKeyPosInf;
        wmax[w][lane] = kKeyNegInf;
    }
    __syncwarp();
    // the chunks of consecutive slots this block takes: its own, or (persistent)
    // the next from the dispenser until none is left
    __shared__ int s_chunk;
    const int nchunks = (n + chunk - 1) / chunk;
    int ck = blockIdx.x;
    if (PERSIST) {
        if (threadIdx.x == 0) s_chunk = (int)atomicAdd(&S.lctl->next_chunk, 1u);
        __syncthreads();
        ck = s_chunk;
    }
    while (ck < nchunks) {
    const int i0 = ck * chunk;
    const int i1 = min(i0 + chunk, n);
    int colony = (i0 + (int)threadIdx.x < i1) ? colony_of(S.cbase, S.ncol, i0 + threadIdx.x) : 0;
    // the first slot of the next colony, kept in a register: the common step
    // compares against it instead of loading it
    int cnext = (colony + 1 < S.ncol) ? __ldg(&S.cbase[colony + 1]) : 0x7fffffff;
    for (int base = i0; base < i1; base += blockDim.x) {  // same trip count for every thread
        const int i = base + threadIdx.x;
        const bool act = i < i1;
        unsigned lo0 = kKeyPosInf, lo1 = kKeyPosInf, lo2 = kKeyPosInf;
        unsigned hi0 = kKeyNegInf, hi1 = kKeyNegInf, hi2 = kKeyNegInf;
        int4 h = make_int4(0, 0, 0, 0);
        int cnt = 0;
        float ux = 0.0f, uy = 0.0f, uz = 0.0f;
        float gx = 0.0f, gy = 0.0f, gz = 0.0f;
        PairRec pr{CAP ? S.pcap : nullptr, i, 0};
        // the pair term: offset from the high words, the gate r < rA, F / r
        auto term = [&](const int4 me, const int4 q, float tx, float ty, float tz, float &ex, float &ey, float &ez,
                        float &Fi) -> bool {
            ex = (float)(me.x - q.x) * tx;
            ey = (float)(me.y - q.y) * ty;
            ez = (float)(me.z - q.z) * tz;
            const float r2f = __fmaf_rn(ex, ex, __fmaf_rn(ey, ey, __fmul_rn(ez, ez)));
            const float rSf = __fadd_rn(__int_as_float(me.w), __int_as_float(q.w));
            const float rAf = __fadd_rn(rSf, bwf);
            if (!(r2f < __fmul_rn(rAf, rAf))) return false;
            const float inv = rsqrtf(r2f);
            const float rn = __fmul_rn(r2f, inv);
            const float d1 = __fsub_rn(rn, rAf);
            const float Fm = __fmul_rn(__fmul_rn(__fmul_rn(-kf, d1), d1), __fsub_rn(rn, rSf));
            Fi = __fmul_rn(Fm, inv);
            return true;
        };
        auto pair = [&](int j, const int4 q) {
            float ex, ey, ez, Fi;
            if (!term(h, q, ux, uy, uz, ex, ey, ez, Fi)) return;
            if (CAP) pr.add(j);
            gx = __fmaf_rn(Fi, ex, gx);
            gy = __fmaf_rn(Fi, ey, gy);
            gz = __fmaf_rn(Fi, ez, gz);
        };
        int4 rec = make_int4(0, 0, 0, 0);
        if (act) {
            while (i >= cnext) {
                ++colony;
                cnext = (colony + 1 < S.ncol) ? __ldg(&S.cbase[colony + 1]) : 0x7fffffff;
            }
            rec = __ldg(&S.lrec[i]);
            h = ga[i];
            cnt = rec.x & 0xff;
            const float4 fu = *reinterpret_cast<const float4 *>(S.fxg[colony].uh);
            ux = fu.x;
            uy = fu.y;
            uz = fu.z;
        }
        if (act) {
            if (cnt <= kNbrCap) {
                // the inline entries: their gathers go out together
                const int4 z4 = make_int4(0, 0, 0, 0);
                const int4 p0 = (cnt > 0) ? __ldg(&ga[rec.y]) : z4;
                const int4 p1 = (cnt > 1) ? __ldg(&ga[rec.z]) : z4;
                const int4 p2 = (cnt > 2) ? __ldg(&ga[rec.w]) : z4;
                if (cnt > 0) pair(rec.y, p0);
                if (cnt > 1) pair(rec.z, p1);
                if (cnt > 2) pair(rec.w, p2);
                // this slot's entries past the inline ones, from its place in
                // its warp's run of the compacted list
                const int xl = list_extra(cnt);
                if (xl) {
                    const int *xs = S.xlist + __ldg(&S.xoff[i >> 5]) + ((rec.x >> 8) & 0x3ff);
                    int k = 0;
                    // four entries in flight at a time: the list loads and the
                    // neighbour gathers are independent across entries
                    for (; k + 4 <= xl; k += 4) {
                        const int e0 = __ldg(xs + k), e1 = __ldg(xs + k + 1);
                        const int e2 = __ldg(xs + k + 2), e3 = __ldg(xs + k + 3);
                        const int4 q0 = __ldg(&ga[e0]);
                        const int4 q1 = __ldg(&ga[e1]);
                        const int4 q2 = __ldg(&ga[e2]);
                        const int4 q3 = __ldg(&ga[e3]);
                        pair(e0, q0);
                        pair(e1, q1);
                        pair(e2, q2);
                        pair(e3, q3);
                    }
                    for (; k < xl; ++k) {
                        const int e = __ldg(xs + k);
                        pair(e, __ldg(&ga[e]));
                    }
                }
            } else {  // list overflow: walk the build's cells with the current records
                const DevGeom &G = S.geoms[colony];
                int bx, by;
                col_to_bxy(G, S.col[B][i], bx, by);
                visit_cells(S, G, S.rank[B][i], bx, by, S.iz[B][i], [&](int s) {
                    const int j = __ldg(&S.perm[B][s]);
                    pair(j, __ldg(&ga[j]));
                });
            }
        }
        if (act) {
            const FxGeom &F = S.fxg[colony];
            if (CAP) pr.done();
            const unsigned zw = F.zw;
            const float ri = __int_as_float(h.w);
            const float dzw = (float)(int)((unsigned)h.z - zw) * uz;
            const float vx = gx, vy = gy, vz = gz + wall_law32(dzw, ri, zkf, zbwf, zgf);
            const float ix = dtf * vx, iy = dtf * vy, iz = dtf * vz;
            bool big = false;
            const float4 fc = *reinterpret_cast<const float4 *>(F.c);
            const float4 fl = *reinterpret_cast<const float4 *>(F.cl);
            const unsigned long long nx =
                fx_join((unsigned)h.x, la[i]) + (unsigned long long)fx_inc(ix, fc.x, fl.x, big);
            const unsigned long long ny =
                fx_join((unsigned)h.y, la[n + i]) + (unsigned long long)fx_inc(iy, fc.y, fl.y, big);
            const unsigned long long nz =
                fx_join((unsigned)h.z, la[2 * (size_t)n + i]) + (unsigned long long)fx_inc(iz, fc.z, fl.z, big);
            const unsigned hz = (unsigned)(nz >> 32);
            // the domain [plo, phi) of a closed axis is the high word in [2^30, 2^31)
            if (hz - (1u << 30) >= (1u << 30)) {
                atomicAdd(&S.cnt->out_of_domain, 1ULL);
                // within three quarters of a length of the domain, or the fixed point's range ends
                if (hz < (1u << 28) || hz >= 0xf0000000u) atomicAdd(&S.cnt->range, 1ULL);
            }
            S.fxh[b][i] = make_int4((int)(nx >> 32), (int)(ny >> 32), (int)hz, h.w);
            unsigned *lb = S.fxl[b];
            lb[i] = (unsigned)nx;
            lb[n + i] = (unsigned)ny;
            lb[2 * (size_t)n + i] = (unsigned)nz;
            S.vxf[i] = vx;
            S.vyf[i] = vy;
            S.vzf[i] = vz;
            lo0 = hi0 = fkey(ix);
            lo1 = hi1 = fkey(iy);
            lo2 = hi2 = fkey(iz);
            if (!isfinite(ix + iy + iz) || big) {
                atomicAdd(&S.cnt->nonfinite, 1ULL);
                lo0 = 0u;  // spreads the bound: the next step rebuilds
                hi0 = 0xffffffffu;
            }
        }
        lo0 = __reduce_min_sync(0xffffffffu, lo0);
        hi0 = __reduce_max_sync(0xffffffffu, hi0);
        lo1 = __reduce_min_sync(0xffffffffu, lo1);
        hi1 = __reduce_max_sync(0xffffffffu, hi1);
        lo2 = __reduce_min_sync(0xffffffffu, lo2);
        hi2 = __reduce_max_sync(0xffffffffu, hi2);
        if (lane == 0) {
            wmin[w][0] = min(wmin[w][0], lo0);
            wmax[w][0] = max(wmax[w][0], hi0);
            wmin[w][1] = min(wmin[w][1], lo1);
            wmax[w][1] = max(wmax[w][1], hi1);
            wmin[w][2] = min(wmin[w][2], lo2);
            wmax[w][2] = max(wmax[w][2], hi2);
        }
    }
    if (!PERSIST) break;
    __syncthreads();  // every thread has read s_chunk
    if (threadIdx.x == 0) s_chunk = (int)atomicAdd(&S.lctl->next_chunk, 1u);
    __syncthreads();
    ck = s_chunk;
    }
    if (PERSIST && threadIdx.x == 0) {
        // the last block to find the dispenser empty resets it for the next launch
        __threadfence();
        if (atomicAdd(&S.lctl->done_blocks, 1u) == gridDim.x - 1) {
            S.lctl->next_chunk = 0u;
            S.lctl->done_blocks = 0u;
            __threadfence();
        }
    }
    // then over the block: six atomics per block, not per warp (updates of
    // one address serialise in its L2 slice)
    __syncthreads();
    if (threadIdx.x < 3) {
        const int k = threadIdx.x;
        unsigned lo = kKeyPosInf, hi = kKeyNegInf;
        for (int v = 0; v < nw; ++v) {
            lo = min(lo, wmin[v][k]);
            hi = max(hi, wmax[v][k]);
        }
        if (hi >= lo) {
            atomicMin(&S.lctl->inc_min[k], lo);
            atomicMax(&S.lctl->inc_max[k], hi);
        }
    }
}

// The two ends of the list path, in integer arithmetic (GB300 issues FP64 at
// a small fraction of the FP32 rate; only an origin other than 0 costs one
// FP64 addition or subtraction per coordinate).
//
// fixed point of a coordinate: (x - o) 2^64 / span, rounded, mod 2^64 on a
// periodic axis, else clamped to the range [0, 2^64) (a closed axis's range
// is four domain lengths from one length below plo).  With d = x - o =
// md 2^ed and 2^64 / span = mc 2^ec the value is md mc 2^(ed + ec): a 117-bit
// product shifted into place.
__device__ __forceinline__ unsigned long long to_fx(double x, const FxGeom &F, int ax)
{
    const double d = F.ozero[ax] ? x : x - F.o[ax];
    const unsigned long long b = (unsigned long long)__double_as_longlong(d);
    const int be = (int)((b >> 52) & 0x7ffu);
    if (be == 0) return 0ull;  // zero (and subnormals)
    const bool neg = (b >> 63) != 0ull;
    const unsigned long long md = (b & 0xfffffffffffffull) | 0x10000000000000ull;
    const unsigned long long hi = __umul64hi(md, F.mc[ax]), lo = md * F.mc[ax];
    const int r = -((be - 1075) + F.ec[ax]);  // X = (hi:lo) >> r
    unsigned long long X;
    bool over = false;
    if (r <= 0) {
        over = true;
        X = 0ull;
    } else if (r < 64) {
        over = (hi >> r) != 0ull;
        X = (hi << (64 - r)) | (lo >> r);
        X += (lo >> (r - 1)) & 1ull;  // round half up
    } else if (r < 128) {
        X = (r == 64) ? hi : (hi >> (r - 64));
        X += (r == 64) ? (lo >> 63) : ((hi >> (r - 65)) & 1ull);
    } else {
        X = 0ull;
    }
    if (F.per[ax]) return neg ? 0ull - X : X;  // the unsigned wrap is the periodic wrap
    if (neg) return 0ull;
    return over ? ~0ull : X;
}

// x of a fixed-point coordinate: o + X span / 2^64, the product X ms 2^(es - 64)
// rounded to nearest even once (then the FP64 addition of a non-zero origin);
// a periodic coordinate is kept below phi.
__device__ __forceinline__ double from_fx(unsigned long long X, const FxGeom &F, int ax)
{
    const unsigned long long ms = F.ms[ax];
    const unsigned long long hi = __umul64hi(X, ms), lo = X * ms;
    unsigned long long t, rest;
    int E;  // value = t 2^E with t in [2^63, 2^64), rest the bits below t
    if (hi) {
        const int lz = __clzll((long long)hi);
        t = lz ? ((hi << lz) | (lo >> (64 - lz))) : hi;
        rest = lo << lz;
        E = F.es[ax] - lz;
    } else if (lo) {
        const int lz = __clzll((long long)lo);
        t = lo << lz;
        rest = 0ull;
        E = F.es[ax] - 64 - lz;
    } else {
        t = 0ull;
        rest = 0ull;
        E = 0;
    }
    double v = 0.0;
    if (t) {
        unsigned long long m = t >> 11;
        const unsigned long long rb = (t >> 10) & 1ull;
        const bool sticky = (t & 0x3ffull) != 0ull || rest != 0ull;
        m += rb & ((sticky ? 1ull : 0ull) | (m & 1ull));
        if (m >> 53) {
            m >>= 1;
            ++E;
        }
        v = __longlong_as_double((long long)((((unsigned long long)(E + 1086)) << 52) | (m & 0xfffffffffffffull)));
    }
    if (F.ozero[ax]) {
        // (periodic with plo = 0: v < len unless rounding reached it)
        if (F.per[ax] && !(v < F.phi[ax])) v = nextafter(F.phi[ax], 0.0);
        return v;
    }
    double x = F.o[ax] + v;
    if (F.per[ax] && !(x < F.phi[ax])) x = nextafter(F.phi[ax], -1.0e300);
    return x;
}

// Fixed-point positions of buffer a from its FP64 positions and the radii
__global__ void k_list_init(const DevState S, int a)
{
    const int n = S.n;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int col = block_colony(S, i);
    if (i < n) {
        const FxGeom &F = S.fxg[col];
        const unsigned long long X = to_fx(S.x[a][i], F, 0);
        const unsigned long long Y = to_fx(S.y[a][i], F, 1);
        const unsigned long long Z = to_fx(S.z[a][i], F, 2);
        S.fxh[a][i] = make_int4((int)(X >> 32), (int)(Y >> 32), (int)(Z >> 32), __float_as_int(d2f_rn(S.rad[i])));
        S.fxl[a][i] = (unsigned)X;
        S.fxl[a][n + i] = (unsigned)Y;
        S.fxl[a][2 * (size_t)n + i] = (unsigned)Z;
    }
}

// FP64 positions of buffer a from its fixed-point positions
__global__ void k_list_to_fp64(const DevState S, int a)
{
    const int n = S.n;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int col = block_colony(S, i);
    if (i < n) {
        const FxGeom &F = S.fxg[col];
        const int4 h = S.fxh[a][i];
        S.x[a][i] = from_fx(fx_join((unsigned)h.x, S.fxl[a][i]), F, 0);
        S.y[a][i] = from_fx(fx_join((unsigned)h.y, S.fxl[a][n + i]), F, 1);
        S.z[a][i] = from_fx(fx_join((unsigned)h.z, S.fxl[a][2 * (size_t)n + i]), F, 2);
    }
}

// One axis of the same conversion, the value also scattered to the caller's
// order (out[orig[i]]): a store of the state converts and gathers in one pass.
__global__ void k_list_to_fp64_axis(const DevState S, int a, int ax, double *out)
{
    const int n = S.n;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int col = block_colony(S, i);
    if (i < n) {
        const FxGeom &F = S.fxg[col];
        const int4 h = S.fxh[a][i];
        const unsigned hi = (unsigned)(ax == 0 ? h.x : (ax == 1 ? h.y : h.z));
        const double v = from_fx(fx_join(hi, S.fxl[a][(size_t)ax * n + i]), F, ax);
        (ax == 0 ? S.x : (ax == 1 ? S.y : S.z))[a][i] = v;
        const int o = S.orig[i];
        if ((unsigned)o < (unsigned)n) out[o] = v;
    }
}

}  // namespace

int launch_list_decide(const DevState &S, unsigned long long cond, int use_cond, cudaStream_t st)
{
    k_list_decide<<<1, 1, 0, st>>>(S.lctl, S.cnt, (cudaGraphConditionalHandle)cond, use_cond);
    return 1;
}

int launch_list_init(const DevState &S, int a, int grid, int block, cudaStream_t st)
{
    (void)grid;  // one slot per thread
    k_list_init<<<(S.n + block - 1) / block, block, 0, st>>>(S, a);
    return 1;
}

int launch_list_to_fp64(const DevState &S, int a, int grid, int block, cudaStream_t st)
{
    (void)grid;  // one slot per thread
    k_list_to_fp64<<<(S.n + block - 1) / block, block, 0, st>>>(S, a);
    return 1;
}

int launch_list_to_fp64_axis(const DevState &S, int a, int ax, double *out, int block, cudaStream_t st)
{
    k_list_to_fp64_axis<<<(S.n + block - 1) / block, block, 0, st>>>(S, a, ax, out);
    return 1;
}

int launch_list_build(const DevState &S, const DevParams &P, int build_block, cudaStream_t st)
{
    k_list_build<<<(S.n + build_block - 1) / build_block, build_block, 0, st>>>(S, P);
    return 1;
}

int launch_list_rebuild(const DevState &S, const DevParams &P, int a, int *scan_scratch, int grid, int block,
                        int build_block, cudaStream_t st)
{
    const int *gate = &S.lctl->rebuild;
    // one slot per thread (a block's colonies from one search)
    const int g1 = (S.n + block - 1) / block;
    k_list_rebin<<<g1, block, 0, st>>>(S, a);
    int k = 1 + launch_scan(S.colcnt, S.colstart[kListBins], S.ncols_total, scan_scratch, st, gate);
    k_list_scatter<<<g1, block, 0, st>>>(S);
    k_list_canon<<<g1, block, 0, st>>>(S, a);
    // the cell offsets: a block per kCellsBlock columns of the largest colony
    const dim3 gc(S.ncol, std::max(1, std::min(65535, (S.cols_max + kCellsBlock - 1) / kCellsBlock)));
    k_list_cells<<<gc, kCellsBlock, 0, st>>>(S);
    // the build: one slot per thread in small blocks (the stencil walks
    // differ in length from slot to slot; small blocks on a grid of every
    // slot let the scheduler balance them)
    launch_list_build(S, P, build_block, st);
    // the entries past the inline ones, compacted per group of 32 slots
    const int gx = (S.n + 127) / 128;
    k = k + launch_scan(S.xcnt, S.xoff, (S.n + 31) / 32, scan_scratch, st, gate);
    k_list_xcopy<<<gx, 128, 0, st>>>(S);
    return k + 5;
}

int launch_list_step(const DevState &S, const DevParams &P, double dt, int a, int grid, int block, int passes,
                     cudaStream_t st, bool persistent)
{
    // passes of the block per chunk (passes <= 0: the rule): short enough that
    // the block scheduler evens out the uneven list lengths of the colonies
    // (one wave of long chunks ends on its slowest block), long enough to
    // amortise the colony search and the block's reduction of the increment
    // spreads.  The rule: two, or one when two would leave fewer than four
    // waves of 1536 threads per SM (grid = the SM count).
    int chunk = block * passes;
    if (passes <= 0) {
        const int two = (S.n + 2 * block - 1) / (2 * block);
        chunk = (two >= 4 * (1536 / block) * grid) ? 2 * block : block;
    }
    const int nb = (S.n + chunk - 1) / chunk;
    if (persistent) {
        // one wave: the blocks that fit on the SMs at once (1536 threads per SM)
        const int wave = std::max(1, std::min(nb, grid * (1536 / block)));
        if (S.pcap) k_list_step<true, true><<<wave, block, 0, st>>>(S, P, (float)dt, a, chunk);
        else k_list_step<false, true><<<wave, block, 0, st>>>(S, P, (float)dt, a, chunk);
    } else {
        if (S.pcap) k_list_step<true, false><<<nb, block, 0, st>>>(S, P, (float)dt, a, chunk);
        else k_list_step<false, false><<<nb, block, 0, st>>>(S, P, (float)dt, a, chunk);
    }
    return 1;
}

}  // namespace bmxg
