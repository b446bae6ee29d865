// k_split.cu -- YEAST cell division on particles in the reference's AoS layout.
//
// BMXParticleContainer::split_particles (src/des/bmx_split_particles.cpp:16-166)
// runs after the DEM step: a flag pass (checkSplit, src/chemistry/bmx_chem_K.H:
// 23-69), an exclusive scan of the flags that gives each dividing cell the slot
// of its daughter past the end of the tile, a read of the total on the host,
// and a fill pass (copyChildParameters + setNewCell, bmx_chem_K.H:357-440).
// Four device passes here:
//   k_split_count  one flag per particle, a count per 256-particle block
//                  (__syncthreads_count), and a flag for FUNGI segments this
//                  build does not divide;
//   k_split_scan   exclusive scan of the block counts in one 1024-thread block
//                  (one count per 256 particles: 10 M particles are 40 k counts);
//   k_split_index  the flags again, a block-local ballot scan on top of the
//                  block's offset: the list of dividing cells in array order;
//   k_split_divide one thread per division of that list.
// The records are read in place (448-byte stride for BMX's 34 reals / 35 ints),
// so the flag passes touch two 32-byte sectors per record; a division copies
// 34 reals and 35 ints of its mother.  Divisions are rare per step (a cell
// divides once per doubling of its volume), so the flag passes dominate.
#include <climits>
#include <cstdint>
#include <cstring>
#include <mutex>

#include <cuda_runtime.h>

#include "../../include/bmxg.h"

namespace bmxg {
namespace {

// realIdx (src/chemistry/bmx_chem.H:38-69)
enum { R_radius = 0, R_c_length = 1, R_area = 4, R_vol = 5, R_dadt = 21, R_dvdt = 22,
       R_bond_scale = 24, R_first = 25 };
// intIdx (src/chemistry/bmx_chem.H:77-118)
enum { I_cell_type = 5, I_position = 19, I_fuse_tip = 25, I_id = 33, I_cpu = 34, I_first = 35 };

constexpr int kBlock = 256;
constexpr int kScanThreads = 1024;

struct SplitArgs {
    unsigned char *par;   // record 0 of the tile
    unsigned char *kid;   // record of daughter 0 (particles + n records, or a staging copy)
    long long n;
    long long stride;     // bytes per record
    int rdata, ids, idata;  // byte offsets of rdata[], (id, cpu), idata[] in a record
    int nreals, nints;    // copied block: reals [0, nreals), ints [0, nints)
    double max_vol, overlap, max_len, max_rad, brnch_prob;
    const double *draws;  // 2 per division, or NULL for the counter generator
    unsigned long long seed;
    long long next_id;
    int my_proc;
    long long *counts;    // [nblocks + 1]: per-block divisions, then their exclusive scan
    unsigned *masks;      // [8 nblocks]: the division flags of each block as ballot words
};

__device__ __forceinline__ double *rec_r(const SplitArgs &a, unsigned char *rec) { return (double *)(rec + a.rdata); }
__device__ __forceinline__ int *rec_i(const SplitArgs &a, unsigned char *rec) { return (int *)(rec + a.idata); }

// 1: a YEAST cell that divides; 2: a FUNGI segment the reference would split or
// branch (checkSplit's FUNGI branches); 0: nothing.
__device__ __forceinline__ int split_kind(const SplitArgs &a, long long i)
{
    unsigned char *rec = a.par + i * a.stride;
    const int *q = rec_i(a, rec);
    const double *r = rec_r(a, rec);
    // both words in flight together: they sit in different sectors of the record
    const int ct = q[I_cell_type];
    const double vol = r[R_vol];
    if (ct == BMXG_YEAST) return vol > a.max_vol ? 1 : 0;
    if (ct == BMXG_FUNGI) {
        const int pos = q[I_position];
        if (pos == BMXG_SITE_TIP)
            return (r[R_radius] >= a.max_rad && r[R_c_length] >= a.max_len) ? 2 : 0;
        if (pos == BMXG_SITE_SECOND_1 || pos == BMXG_SITE_SECOND_2) return a.brnch_prob > 0.0 ? 2 : 0;
    }
    return 0;
}

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

// per 256-particle block: the division flags as 8 ballot words, and the count
// (or -1 when the block holds a FUNGI segment that would split or branch)
__global__ void __launch_bounds__(kBlock) k_split_count(SplitArgs a)
{
    const long long i = (long long)blockIdx.x * kBlock + threadIdx.x;
    const int kind = i < a.n ? split_kind(a, i) : 0;
    const unsigned b = __ballot_sync(0xffffffffu, kind == 1);
    if ((threadIdx.x & 31) == 0) a.masks[(long long)blockIdx.x * (kBlock / 32) + (threadIdx.x >> 5)] = b;
    const int cnt = __syncthreads_count(kind == 1);
    const int bad = __syncthreads_or(kind == 2);
    if (threadIdx.x == 0) a.counts[blockIdx.x] = bad ? -1 : cnt;
}

// exclusive scan of counts[0, nb) in place; counts[nb] = the total, or -1
// when a block reported a FUNGI segment outside the YEAST division
__global__ void __launch_bounds__(kScanThreads) k_split_scan(long long *counts, int nb)
{
    __shared__ long long s[kScanThreads];
    __shared__ int bad;
    const int t = threadIdx.x;
    if (t == 0) bad = 0;
    __syncthreads();
    const int per = (nb + kScanThreads - 1) / kScanThreads;
    const long long lo = (long long)t * per;
    const long long hi = lo + per < nb ? lo + per : nb;
    long long sum = 0;
    int neg = 0;
    for (long long j = lo; j < hi; ++j) {
        const long long v = counts[j];
        neg |= v < 0;
        sum += v < 0 ? 0 : v;
    }
    if (neg) bad = 1;
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
        const long long v = counts[j];
        counts[j] = run;
        run += v < 0 ? 0 : v;
    }
    if (t == kScanThreads - 1) counts[nb] = bad ? -1 : s[t];
}

// copyChildParameters + setNewCell (bmx_chem_K.H:357-440) for division k of
// cell i, after the copy of the mother's block into the daughter (done by the
// warp, k_split_divide), then the identity the caller loop gives the daughter
// (bmx_split_particles.cpp:95-121).  The expressions keep the reference's
// order and grouping; the library is built without FMA contraction.
__device__ void divide(const SplitArgs &a, long long i, long long k)
{
    unsigned char *mrec = a.par + i * a.stride;
    unsigned char *drec = a.kid + k * a.stride;
    double *mp = (double *)mrec, *dp = (double *)drec;
    double *mr = rec_r(a, mrec), *dr = rec_r(a, drec);
    int *di = rec_i(a, drec);
    const int *mid = (const int *)(mrec + a.ids);
    int *did = (int *)(drec + a.ids);

    double u1, u2;
    if (a.draws) {
        u1 = a.draws[2 * k];
        u2 = a.draws[2 * k + 1];
    } else {
        u1 = split_uniform(a.seed, mid[0], mid[1], 0);
        u2 = split_uniform(a.seed, mid[0], mid[1], 1);
    }
    const double x = mp[0], y = mp[1], z = mp[2];
    double radius = mr[R_radius];
    double theta = 2.0 * u1 - 1.0;
    theta = acos(theta);
    const double phi = 2.0 * M_PI * u2;
    double st, ct, sp, cp;
    sincos(theta, &st, &ct);
    sincos(phi, &sp, &cp);
    const double nx = st * cp;
    const double ny = st * sp;
    const double nz = ct;
    const double scale = 1.0 - a.overlap;
    dp[0] = x + scale * 0.5 * nx * radius;
    dp[1] = y + scale * 0.5 * ny * radius;
    dp[2] = z + scale * 0.5 * nz * radius;
    mp[0] = x - scale * 0.5 * nx * radius;
    mp[1] = y - scale * 0.5 * ny * radius;
    mp[2] = z - scale * 0.5 * nz * radius;

    const double volume = mr[R_vol] / 2.0;
    radius = pow((3.0 * volume / (4.0 * M_PI)), 1.0 / 3.0);
    const double area = 4.0 * M_PI * radius * radius;
    const double dvdt = mr[R_dvdt];
    const double dadt = 2.0 * dvdt / radius;
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

    const int new_id = (int)(a.next_id + k);
    did[0] = new_id;
    did[1] = a.my_proc;
    di[I_id] = new_id;
    di[I_cpu] = a.my_proc;
}

// the dividing cells in array order, list[k] = i for division k, from the
// count pass's ballot words (the records are not read again)
__global__ void __launch_bounds__(kBlock) k_split_index(SplitArgs a, int *list)
{
    __shared__ int wsum[kBlock / 32];
    const long long i = (long long)blockIdx.x * kBlock + threadIdx.x;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned b = a.masks[(long long)blockIdx.x * (kBlock / 32) + w];
    if (lane == 0) wsum[w] = __popc(b);
    __syncthreads();
    if (!((b >> lane) & 1u)) return;
    int off = __popc(b & ((1u << lane) - 1u));
    for (int j = 0; j < w; ++j) off += wsum[j];
    list[a.counts[blockIdx.x] + off] = (int)i;
}

// One thread per division over the compacted list, so that the FP64 acos /
// sin / cos / pow of a division run with full warps (a few percent of the
// cells divide in a step; one thread per cell would leave most lanes idle).
// First the warp copies the copied block (copyChildParameters) of its 32
// mothers into their daughters: the (record, word) pairs are spread over the
// lanes, kCopyUnroll loads in flight per lane before their stores, so the copy
// costs a few memory round trips rather than one per record.  Small blocks
// (kDivBlock): a step divides a few thousand cells, which must still cover
// every SM.
constexpr int kDivBlock = 64;
constexpr int kCopyUnroll = 8;

template <typename T>
__device__ __forceinline__ void copy_block(const SplitArgs &a, const int *mothers, long long k0, int nk, int lane,
                                           int nwords, int off)
{
    const int total = nk * nwords;
    for (int t0 = lane; t0 < total; t0 += 32 * kCopyUnroll) {
        T v[kCopyUnroll];
#pragma unroll
        for (int u = 0; u < kCopyUnroll; ++u) {
            const int t = t0 + 32 * u;
            if (t < total) {
                const int j = t / nwords, w = t - j * nwords;
                v[u] = ((const T *)(a.par + (long long)mothers[j] * a.stride + off))[w];
            }
        }
#pragma unroll
        for (int u = 0; u < kCopyUnroll; ++u) {
            const int t = t0 + 32 * u;
            if (t < total) {
                const int j = t / nwords, w = t - j * nwords;
                ((T *)(a.kid + (k0 + j) * a.stride + off))[w] = v[u];
            }
        }
    }
}

__global__ void __launch_bounds__(kDivBlock) k_split_divide(SplitArgs a, const int *list, long long total)
{
    __shared__ int mothers[kDivBlock];
    const long long k0 = (long long)blockIdx.x * kDivBlock + (threadIdx.x & ~31);
    if (k0 >= total) return;
    const int lane = threadIdx.x & 31;
    const long long k = k0 + lane;
    const int mine = k < total ? list[k] : 0;
    int *wm = mothers + (threadIdx.x & ~31);
    wm[lane] = mine;
    __syncwarp();
    const int nk = total - k0 < 32 ? (int)(total - k0) : 32;
    copy_block<double>(a, wm, k0, nk, lane, a.nreals, a.rdata);
    copy_block<int>(a, wm, k0, nk, lane, a.nints, a.idata);
    __syncwarp();
    if (k < total) divide(a, mine, k);
}

// Per-device scratch kept across calls (the division list, the block counts
// and ballot words, and a pinned word for the host's read of the total); it
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
    if (n > INT_MAX) return BMXG_ERR_ARG;  // the reference's particle index is an int
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
    a.seed = seed;
    a.next_id = next_id;
    a.my_proc = my_proc;

    cudaStream_t st = static_cast<cudaStream_t>(stream);
    DevScratch &S = g_scratch[dev];
    std::lock_guard<std::mutex> lock(S.mu);
    const long long nb = (n + kBlock - 1) / kBlock;
    // counts [nb + 1] (8-byte), ballot words [8 nb], the list [n] (at most n divisions)
    const size_t off_masks = sizeof(long long) * (size_t)(nb + 1);
    const size_t off_list = off_masks + sizeof(unsigned) * (size_t)nb * (kBlock / 32);
    const size_t need = off_list + sizeof(int) * (size_t)n;
    if (!S.host) SPLIT_CK(cudaMallocHost((void **)&S.host, sizeof(long long)));
    if (S.dev_bytes < need) {
        SPLIT_CK(cudaStreamSynchronize(st));
        if (S.dev) SPLIT_CK(cudaFree(S.dev));
        S.dev = nullptr;
        S.dev_bytes = 0;
        if (cudaMalloc((void **)&S.dev, need) != cudaSuccess) return BMXG_ERR_OOM;
        S.dev_bytes = need;
    }
    a.counts = (long long *)S.dev;
    a.masks = (unsigned *)(S.dev + off_masks);
    int *list = (int *)(S.dev + off_list);

    Staging stage(st);
    const size_t rec_bytes = (size_t)n * (size_t)a.stride;
    if (where == BMXG_DEVICE) {
        a.par = static_cast<unsigned char *>(particles);
    } else {
        a.par = (unsigned char *)stage.get(rec_bytes);
        if (!a.par) return BMXG_ERR_OOM;
        SPLIT_CK(cudaMemcpyAsync(a.par, particles, rec_bytes, cudaMemcpyHostToDevice, st));
    }

    k_split_count<<<(unsigned)nb, kBlock, 0, st>>>(a);
    k_split_scan<<<1, kScanThreads, 0, st>>>(a.counts, (int)nb);
    SPLIT_CK(cudaGetLastError());
    SPLIT_CK(cudaMemcpyAsync(S.host, a.counts + nb, sizeof(long long), cudaMemcpyDeviceToHost, st));
    SPLIT_CK(cudaStreamSynchronize(st));
    const long long total = *S.host;
    if (total < 0) return BMXG_ERR_UNSUPPORTED;
    *num_split = total;
    if (total == 0) return BMXG_OK;
    if (n + total > cap) return BMXG_ERR_CAPACITY;
    if (draws && ndraws < 2 * total) return BMXG_ERR_ARG;

    unsigned char *host_kids = static_cast<unsigned char *>(particles) + rec_bytes;
    const size_t kid_bytes = (size_t)total * (size_t)a.stride;
    if (where == BMXG_DEVICE) {
        a.kid = a.par + rec_bytes;
        a.draws = draws;
    } else {
        // the daughters' records start from what the caller's buffer holds, so
        // the fields a division leaves unset come back unchanged
        a.kid = (unsigned char *)stage.get(kid_bytes);
        if (!a.kid) return BMXG_ERR_OOM;
        SPLIT_CK(cudaMemcpyAsync(a.kid, host_kids, kid_bytes, cudaMemcpyHostToDevice, st));
        if (draws) {
            double *d = (double *)stage.get(sizeof(double) * 2 * (size_t)total);
            if (!d) return BMXG_ERR_OOM;
            SPLIT_CK(cudaMemcpyAsync(d, draws, sizeof(double) * 2 * (size_t)total, cudaMemcpyHostToDevice, st));
            a.draws = d;
        }
    }
    k_split_index<<<(unsigned)nb, kBlock, 0, st>>>(a, list);
    k_split_divide<<<(unsigned)((total + kDivBlock - 1) / kDivBlock), kDivBlock, 0, st>>>(a, list, total);
    SPLIT_CK(cudaGetLastError());
    if (where == BMXG_HOST) {
        SPLIT_CK(cudaMemcpyAsync(particles, a.par, rec_bytes, cudaMemcpyDeviceToHost, st));
        SPLIT_CK(cudaMemcpyAsync(host_kids, a.kid, kid_bytes, cudaMemcpyDeviceToHost, st));
    }
    SPLIT_CK(cudaStreamSynchronize(st));
    return BMXG_OK;
}
