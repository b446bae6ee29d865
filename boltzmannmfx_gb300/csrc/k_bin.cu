// k_bin.cu -- counting-sort binning of the slots into columns, the prefix
// scan, the deterministic in-column order, the caller-order <-> slot-order
// moves, and the neighbour-list export.
//
// Replaces AMReX's neighbour machinery as BMX drives it every step
// (clearNeighbors / Redistribute / fillNeighbors / buildNeighborList,
// src/des/bmx_pc_interaction.cpp:97-103): bins are the level's cells, the
// pair predicate is BMXCheckPair(DEM::neighborhood, false)
// (src/des/bmx_pc.H:55-82), periodic images come from a one-cell halo
// (src/des/bmx_pc.cpp:23).  All of it is integer / byte work bounded by HBM
// and L2 bandwidth; nothing here is a contraction.
#include "bmxg_stencil.cuh"

namespace bmxg {

namespace {

__global__ void k_bin(const DevState S, int b)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < S.n; i += gridDim.x * blockDim.x) {
        const DevGeom &G = geom_of(S, i);
        rebin_slot(S, G, i, S.x[b][i], S.y[b][i], S.z[b][i], S.rad[i], b);
    }
}

// ---- exclusive scan of n ints into n+1 offsets ----------------------------
// Three passes: tile sums, a scan of the tile sums, the scan of each tile with
// its offset.  A thread holds four consecutive counts, read and written as one
// 16-byte vector (coalesced across the warp); a tile is 1024 counts.
constexpr int kScanBlock = 256;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanBlock * kScanItems;

__device__ __forceinline__ int block_exclusive_scan(int v, int &total)
{
    __shared__ int warp_sums[kScanBlock / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int w = (lane < kScanBlock / 32) ? warp_sums[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < kScanBlock / 32) warp_sums[lane] = w;
    }
    __syncthreads();
    const int before = (warp > 0) ? warp_sums[warp - 1] : 0;
    total = warp_sums[kScanBlock / 32 - 1];
    __syncthreads();
    return before + x - v;
}

// this thread's four counts (zero past n): one vector load where all four lie inside
__device__ __forceinline__ int4 scan_load4(const int *__restrict__ in, int n, int base)
{
    if (base + 3 < n) return __ldg(reinterpret_cast<const int4 *>(in + base));
    int4 v = make_int4(0, 0, 0, 0);
    if (base < n) v.x = in[base];
    if (base + 1 < n) v.y = in[base + 1];
    if (base + 2 < n) v.z = in[base + 2];
    return v;
}

__global__ void k_scan_reduce(const int *__restrict__ in, int n, int *__restrict__ bsum, const int *gate)
{
    if (gate && !*gate) return;
    const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    const int4 v = scan_load4(in, n, base);
    int total;
    block_exclusive_scan(v.x + v.y + v.z + v.w, total);
    if (threadIdx.x == 0) bsum[blockIdx.x] = total;
}

// one block of 1024 threads over the nb tile sums: each thread sums a
// contiguous segment (its loads independent of each other), one block-wide
// scan joins the segments, each thread writes its segment's offsets
constexpr int kTopBlock = 1024;

__global__ void __launch_bounds__(kTopBlock) k_scan_top(int *bsum, int nb, const int *gate)
{
    if (gate && !*gate) return;
    __shared__ int warp_sums[kTopBlock / 32];
    const int seg = (nb + kTopBlock - 1) / kTopBlock;
    const int b0 = min((int)threadIdx.x * seg, nb), b1 = min(b0 + seg, nb);
    int s = 0;
#pragma unroll 8
    for (int k = b0; k < b1; ++k) s += bsum[k];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int w = warp_sums[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        warp_sums[lane] = w;
    }
    __syncthreads();
    int run = ((warp > 0) ? warp_sums[warp - 1] : 0) + x - s;
    for (int k = b0; k < b1; ++k) {
        const int v = bsum[k];
        bsum[k] = run;
        run += v;
    }
    if (threadIdx.x == 0) bsum[nb] = warp_sums[kTopBlock / 32 - 1];
}

__global__ void k_scan_apply(const int *__restrict__ in, int n, const int *__restrict__ bsum,
                             int *__restrict__ out, const int *gate)
{
    if (gate && !*gate) return;
    const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    const int4 v = scan_load4(in, n, base);
    int total;
    const int run = block_exclusive_scan(v.x + v.y + v.z + v.w, total) + bsum[blockIdx.x];
    const int4 o = make_int4(run, run + v.x, run + v.x + v.y, run + v.x + v.y + v.z);
    if (base + 3 < n) {
        *reinterpret_cast<int4 *>(out + base) = o;
    } else {
        if (base < n) out[base] = o.x;
        if (base + 1 < n) out[base + 1] = o.y;
        if (base + 2 < n) out[base + 2] = o.z;
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) out[n] = bsum[gridDim.x];
}

// ---- scatter into columns, then the deterministic in-column order --------
// Arrival order from the atomics is arbitrary; k_canon ranks every slot by
// its (z bin, original index) key among the members of its column, which is
// the order AMReX's serial binning gives (ascending index within a bin).
// With key scratch (S.lkey: a context's state) the scatter leaves each slot's
// key at the position it drew and the rank is counted over the column's keys;
// without it (a bare caller's scratch) the slot index goes there and the
// rank gathers each member's key.
__global__ void k_scatter(const DevState S, int b, const int *gate)
{
    if (gate && !*gate) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < S.n; i += gridDim.x * blockDim.x) {
        const int c = S.col[b][i];
        const int r = atomicSub(&S.colcnt[c], 1) - 1;  // leaves colcnt at zero
        const int t = S.colstart[b][c] + r;
        if (t >= 0 && t < S.n) {
            if (S.lkey) S.lkey[t] = col_key(S.iz[b][i], S.orig[i]);
            else S.tmp[t] = i;
        } else {
            atomicAdd(&S.cnt->bad_index, 1ULL);
        }
    }
}

__global__ void k_canon(const DevState S, int b, int ra, const int *gate)
{
    if (gate && !*gate) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < S.n; i += gridDim.x * blockDim.x) {
        const int c = S.col[b][i];
        const int s0 = max(S.colstart[b][c], 0), s1 = min(S.colstart[b][c + 1], S.n);
        const int izi = S.iz[b][i];
        const unsigned long long key = col_key(izi, S.orig[i]);
        int rank = 0;
        if (S.lkey) {
            for (int t = s0; t < s1; ++t) rank += (__ldg(&S.lkey[t]) < key);
        } else {
            for (int t = s0; t < s1; ++t) {
                const int j = S.tmp[t];
                if ((unsigned)j < (unsigned)S.n) rank += (col_key(S.iz[b][j], S.orig[j]) < key);
            }
        }
        const int t = s0 + rank;
        if (t >= s1) {  // i is not among its column's members: inconsistent counts
            atomicAdd(&S.cnt->bad_index, 1ULL);
            continue;
        }
        S.perm[b][t] = i;
        if (S.srel[b]) {
            S.srel[b][t] = S.rel[ra][i];
            S.siz[b][t] = izi;
            S.rank[b][i] = t;
        }
    }
}

// caller-order variants used once by set_state (orig == caller index)
__global__ void k_user_bin(const DevState S, const double *ux, const double *uy, const double *uz,
                           int *ucol, int *uiz)
{
    for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < S.n; u += gridDim.x * blockDim.x) {
        const DevGeom &G = geom_of(S, u);  // colony slot ranges equal caller ranges
        const int bx = bin_of_fast(ux[u], G.plo[0], G.dxi[0], G.plof[0], G.dxif[0], 1, G.n[0]);
        const int by = bin_of_fast(uy[u], G.plo[1], G.dxi[1], G.plof[1], G.dxif[1], 1, G.n[1]);
        const int bz = bin_of_fast(uz[u], G.plo[2], G.dxi[2], G.plof[2], G.dxif[2], 1, G.n[2]);
        const int c = column_of(G, bx, by);
        ucol[u] = c;
        uiz[u] = bz;
        atomicAdd(&S.colcnt[c], 1);
    }
}

// counting sort of the caller's particles into the columns (arrival order
// from the atomics): each particle's (z bin, caller index) key at the
// position it drew
__global__ void k_user_scatter(const DevState S, const int *ucol, const int *uiz, const int *colstart)
{
    for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < S.n; u += gridDim.x * blockDim.x) {
        const int c = ucol[u];
        const int r = atomicSub(&S.colcnt[c], 1) - 1;
        const int t = colstart[c] + r;
        if (t >= 0 && t < S.n) S.lkey[t] = col_key(uiz[u], u);
        else atomicAdd(&S.cnt->bad_index, 1ULL);
    }
}

__global__ void k_gather_d(double *dst, const double *src, const int *perm, int n)
{
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x)
        dst[s] = src[perm[s]];
}

__global__ void k_gather_i(int *dst, const int *src, const int *perm, int n, int planes)
{
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
        const int u = perm[s];
        for (int k = 0; k < planes; ++k) dst[(size_t)k * n + s] = src[(size_t)k * n + u];
    }
}

__global__ void k_scatter_d(double *dst, const double *src, const int *orig, int n)
{
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x)
        dst[orig[s]] = src[s];
}

__global__ void k_scatter_f2d(double *dst, const float *src, const int *orig, int n)
{
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x)
        dst[orig[s]] = (double)src[s];
}

__global__ void k_scatter_i(int *dst, const int *src, const int *orig, int n, int planes)
{
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
        const int u = orig[s];
        for (int k = 0; k < planes; ++k) dst[(size_t)k * n + u] = src[(size_t)k * n + s];
    }
}

__global__ void k_trig(const DevState S, int b)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < S.n; i += gridDim.x * blockDim.x) {
        const double th = S.theta[b][i], ph = S.phi[b][i];
        double st, ct, sp, cp;
        sincos(th, &st, &ct);
        sincos(ph, &sp, &cp);
        S.trig[b][i] = make_trig(ct, st, cp, sp);
    }
}

// Neighbour list of every slot in the reference's order; indices and counts
// are in caller order.  Only pairs passing BMXCheckPair (|r|^2 <= neighborhood,
// evaluated in FP64 on the image positions) are listed.
__global__ void k_pairs(const DevState S, const DevParams P, int a, int64_t *cnt_or_offs, int *idx,
                        int8_t *img, int mode)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < S.n; i += gridDim.x * blockDim.x) {
        const DevGeom &G = geom_of(S, i);
        int bx, by;
        col_to_bxy(G, S.col[a][i], bx, by);
        const double xi = S.x[a][i], yi = S.y[a][i], zi = S.z[a][i];
        int64_t o = (mode == 1) ? cnt_or_offs[S.orig[i]] : 0;
        int64_t c = 0;
        visit_stencil(S, G, a, i, bx, by, S.iz[a][i], [&](int j, int, int, int, int sx, int sy) {
            const double xj = sx ? S.x[a][j] + (double)sx * G.len[0] : S.x[a][j];
            const double yj = sy ? S.y[a][j] + (double)sy * G.len[1] : S.y[a][j];
            const double dx = xi - xj, dy = yi - yj, dz = zi - S.z[a][j];
            const double r2 = dx * dx + dy * dy + dz * dz;
            if (r2 <= P.nbh) {
                if (mode == 1) {
                    idx[o] = S.orig[j];
                    img[o] = (int8_t)((sx + 1) + 3 * (sy + 1));
                    ++o;
                }
                ++c;
            }
        });
        if (mode == 0) cnt_or_offs[S.orig[i]] = c;
    }
}

// Checks of a caller's state before it is loaded: cell types outside
// {YEAST, FUNGI}, whether any FUNGI segment is present, the largest radius
// (non-negative doubles order as their bit patterns) and whether any radius
// is NaN.  out: {bad, fungi, rmax bits, nan}, zeroed by the caller.
// Whether a load repeats the device state bit for bit: each slot's position
// (buffer a), radius and cell type against the caller's arrays at its caller
// index.  *diff becomes nonzero on the first difference.
__global__ void k_same_state(const DevState S, int a, const double *__restrict__ x, const double *__restrict__ y,
                             const double *__restrict__ z, const double *__restrict__ r, const int *__restrict__ ct,
                             unsigned long long *diff)
{
    unsigned d = 0;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < S.n; s += gridDim.x * blockDim.x) {
        const int i = S.orig[s];
        if ((unsigned)i >= (unsigned)S.n) {
            d = 1u;
            continue;
        }
        // (a null field is not compared: a load compares each field as its copy lands)
        if (x) d |= (__double_as_longlong(x[i]) != __double_as_longlong(S.x[a][s])) ? 1u : 0u;
        if (y) d |= (__double_as_longlong(y[i]) != __double_as_longlong(S.y[a][s])) ? 1u : 0u;
        if (z) d |= (__double_as_longlong(z[i]) != __double_as_longlong(S.z[a][s])) ? 1u : 0u;
        if (r) d |= (__double_as_longlong(r[i]) != __double_as_longlong(S.rad[s])) ? 1u : 0u;
        if (ct) d |= (ct[i] != (int)S.ctype[s]) ? 1u : 0u;
    }
    d = __reduce_or_sync(0xffffffffu, d);
    if ((threadIdx.x & 31) == 0 && d) atomicOr(diff, 1ull);
}

__global__ void k_check_state(const int *__restrict__ ct, const double *__restrict__ r, int n,
                              unsigned long long *out)
{
    unsigned bad = 0, fungi = 0, nan = 0;
    unsigned long long rmax = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const unsigned c = (unsigned)ct[i];
        bad |= (c > 1u) ? 1u : 0u;
        fungi |= (c == 1u) ? 1u : 0u;
        const double v = r[i];
        nan |= (v != v) ? 1u : 0u;
        if (v > 0.0) rmax = max(rmax, (unsigned long long)__double_as_longlong(v));
    }
    bad = __reduce_or_sync(0xffffffffu, bad);
    fungi = __reduce_or_sync(0xffffffffu, fungi);
    nan = __reduce_or_sync(0xffffffffu, nan);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) rmax = max(rmax, __shfl_xor_sync(0xffffffffu, rmax, o));
    if ((threadIdx.x & 31) == 0) {
        if (bad) atomicOr(&out[0], 1ull);
        if (fungi) atomicOr(&out[1], 1ull);
        if (rmax) atomicMax(&out[2], rmax);
        if (nan) atomicOr(&out[3], 1ull);
    }
}

// Caller particle u's slot: its column's start + its rank among the
// column's keys (z bin, then caller index): uperm[slot] = u.
__global__ void k_user_canon(const DevState S, const int *ucol, const int *uiz, const int *colstart, int *uperm)
{
    for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < S.n; u += gridDim.x * blockDim.x) {
        const int c = ucol[u];
        const int s0 = max(colstart[c], 0), s1 = min(colstart[c + 1], S.n);
        const unsigned long long key = col_key(uiz[u], u);
        int rank = 0;
        for (int t = s0; t < s1; ++t) rank += (__ldg(&S.lkey[t]) < key);
        if (s0 + rank < s1) uperm[s0 + rank] = u;
        else atomicAdd(&S.cnt->bad_index, 1ULL);
    }
}

// Slot s of a freshly sorted state holds caller particle uperm[s]: its
// position, radius and cell type are gathered from the caller-order arrays,
// its bins are the caller-order bins of the sort, its column order is the
// sort's (perm = identity, colstart = the sort's offsets, copied by the
// caller), and its offsets and counters are place_slot's.
__global__ void k_load_slots(const DevState S, const double *ux, const double *uy, const double *uz,
                             const double *ur, const int *uct, const int *ucol, const int *uiz, const int *uperm)
{
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < S.n; s += gridDim.x * blockDim.x) {
        const DevGeom &G = geom_of(S, s);
        const int u = uperm[s];
        const double x = ux[u], y = uy[u], z = uz[u], r = ur[u];
        S.x[0][s] = x;
        S.y[0][s] = y;
        S.z[0][s] = z;
        S.rad[s] = r;
        S.ctype[s] = (int8_t)uct[u];
        S.orig[s] = u;
        int bx, by;
        col_to_bxy(G, ucol[u], bx, by);
        const int bz = uiz[u];
        place_slot(S, G, s, x, y, z, r, 0, 0, bx, by, bz, true, false);
        S.perm[0][s] = s;
        if (S.srel[0]) {
            S.srel[0][s] = S.rel[0][s];
            S.siz[0][s] = bz;
            S.rank[0][s] = s;
        }
    }
}

}  // namespace

int launch_load_slots(const DevState &S, const double *ux, const double *uy, const double *uz, const double *ur,
                      const int *uct, const int *ucol, const int *uiz, const int *uperm, int grid, int block,
                      cudaStream_t st)
{
    k_load_slots<<<grid, block, 0, st>>>(S, ux, uy, uz, ur, uct, ucol, uiz, uperm);
    return 1;
}

int launch_check_state(const int *ct, const double *r, int n, unsigned long long *out, int grid, int block,
                       cudaStream_t st)
{
    k_check_state<<<grid, block, 0, st>>>(ct, r, n, out);
    return 1;
}

int launch_same_state(const DevState &S, int a, const double *x, const double *y, const double *z, const double *r,
                      const int *ct, unsigned long long *diff, int grid, int block, cudaStream_t st)
{
    k_same_state<<<grid, block, 0, st>>>(S, a, x, y, z, r, ct, diff);
    return 1;
}

int launch_bin(const DevState &S, int b, int grid, int block, cudaStream_t st)
{
    k_bin<<<grid, block, 0, st>>>(S, b);
    return 1;
}

size_t scan_scratch_ints(int n)
{
    return (size_t)((n + kScanTile - 1) / kScanTile) + 2;
}

int launch_scan(const int *in, int *out, int n, int *scratch, cudaStream_t st, const int *gate)
{
    const int nb = (n + kScanTile - 1) / kScanTile;
    if (nb == 0) {
        cudaMemsetAsync(out, 0, sizeof(int), st);
        return 0;
    }
    k_scan_reduce<<<nb, kScanBlock, 0, st>>>(in, n, scratch, gate);
    k_scan_top<<<1, kTopBlock, 0, st>>>(scratch, nb, gate);
    k_scan_apply<<<nb, kScanBlock, 0, st>>>(in, n, scratch, out, gate);
    return 3;
}

int launch_scatter_canon(const DevState &S, int b, int grid, int block, cudaStream_t st, int ra, const int *gate)
{
    k_scatter<<<grid, block, 0, st>>>(S, b, gate);
    k_canon<<<grid, block, 0, st>>>(S, b, ra < 0 ? b : ra, gate);
    return 2;
}

int launch_rebuild(const DevState &S, int b, int *scan_scratch, int grid, int block, cudaStream_t st, int ra,
                   const int *gate)
{
    int k = launch_scan(S.colcnt, S.colstart[b], S.ncols_total, scan_scratch, st, gate);
    return k + launch_scatter_canon(S, b, grid, block, st, ra, gate);
}

int launch_user_bin(const DevState &S, const double *ux, const double *uy, const double *uz, int *ucol,
                     int *uiz, int grid, int block, cudaStream_t st)
{
    k_user_bin<<<grid, block, 0, st>>>(S, ux, uy, uz, ucol, uiz);
    return 1;
}

int launch_user_scatter_canon(const DevState &S, const int *ucol, const int *uiz, const int *colstart,
                               int *uperm, int grid, int block, cudaStream_t st)
{
    k_user_scatter<<<grid, block, 0, st>>>(S, ucol, uiz, colstart);
    k_user_canon<<<grid, block, 0, st>>>(S, ucol, uiz, colstart, uperm);
    return 2;
}

int launch_gather_d(double *dst, const double *src, const int *perm, int n, int grid, int block,
                     cudaStream_t st)
{
    k_gather_d<<<grid, block, 0, st>>>(dst, src, perm, n);
    return 1;
}

int launch_gather_i(int *dst, const int *src, const int *perm, int n, int planes, int grid, int block,
                     cudaStream_t st)
{
    k_gather_i<<<grid, block, 0, st>>>(dst, src, perm, n, planes);
    return 1;
}

int launch_scatter_d(double *dst, const double *src, const int *orig, int n, int grid, int block,
                      cudaStream_t st)
{
    k_scatter_d<<<grid, block, 0, st>>>(dst, src, orig, n);
    return 1;
}

int launch_scatter_f2d(double *dst, const float *src, const int *orig, int n, int grid, int block,
                       cudaStream_t st)
{
    k_scatter_f2d<<<grid, block, 0, st>>>(dst, src, orig, n);
    return 1;
}

int launch_scatter_i(int *dst, const int *src, const int *orig, int n, int planes, int grid, int block,
                      cudaStream_t st)
{
    k_scatter_i<<<grid, block, 0, st>>>(dst, src, orig, n, planes);
    return 1;
}

int launch_trig(const DevState &S, int b, int grid, int block, cudaStream_t st)
{
    k_trig<<<grid, block, 0, st>>>(S, b);
    return 1;
}

int launch_pairs(const DevState &S, const DevParams &P, int a, int64_t *cnt_or_offs, int *idx, int8_t *img,
                  int mode, int grid, int block, cudaStream_t st)
{
    k_pairs<<<grid, block, 0, st>>>(S, P, a, cnt_or_offs, idx, img, mode);
    return 1;
}

}  // namespace bmxg
