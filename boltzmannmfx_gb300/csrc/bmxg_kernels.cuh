// bmxg_kernels.cuh -- device state of a context and the host launchers of
// every kernel (internal to libbmxg; the public surface is include/bmxg.h).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "bmxg_dev.cuh"

namespace bmxg {

__host__ __device__ __forceinline__ double4_32a make_trig(double ct, double st, double cp, double sp)
{
    double4_32a t;
    t.x = ct;
    t.y = st;
    t.z = cp;
    t.w = sp;
    return t;
}

// Control block of the FP32F neighbour list with a skin (k_list.cu).  The
// list stays valid while no pair's separation has changed by the skin since
// it was built; acc bounds that change from above.
struct ListCtl {
    // per component, the smallest and largest position increment of the last
    // step over all slots (order-preserving integer keys of the floats); the
    // change of any pair's separation since the build is bounded per
    // component by the sum over steps of (largest - smallest)
    unsigned inc_min[3], inc_max[3];
    float range[3];        // those sums since the last build
    float acc;             // |range|: the bound on any pair's separation change
    float skin;            // list skin (cm)
    float eps_step;        // FP32 rounding of one position update, added per step
    int age;               // steps since the last build
    int max_age;           // rebuild at least this often (bounds FP32 offset drift)
    int force;             // rebuild at the next step (the state changed)
    int rebuild;           // this step's decision (read by the gated kernels)
    int builds;            // builds decided so far
    unsigned long long body_runs;  // builds actually run (counted by the first build kernel)
    unsigned long long overflow;   // slots whose list exceeded the capacity (last build)
    // the persistent list step's chunk dispenser: the next chunk to hand out
    // and the blocks that found none left; the last of them resets both
    unsigned next_chunk, done_blocks;
};

constexpr int kNbrCap = 32;          // list entries per slot (more: the slot walks its stencil)
constexpr int kNbrInline = 3;        // entries held in the slot's list record beside its metadata
constexpr int kNbrShift = 31;        // entries are slots below 2^31
constexpr int kPairCap = 32;         // gated pairs per slot the step records when asked
constexpr int kListBins = 0;         // list mode keeps its frozen bins in buffer 0
constexpr int kListStepBlock = 128;  // k_list_step's default block (at most 256; autotuned)
constexpr int kListBuildBlock = 128; // k_list_build's default block (one slot per thread; at most 256)
constexpr int kSphereBlock = 64;     // per-step sphere kernels' block (one slot per thread)
constexpr int kRodCap = 32;          // gated pairs per segment the FP32F rod pipeline holds (more: the
                                     // segment walks its stencil in the segment kernel)

// Per-step counters of the FP32F rod pipeline (k_rod.cu).
struct RodCtl {
    int kmax;   // largest number of gated pairs of a segment (at most kRodCap)
    int nwork;  // pairs queued for FP64
};

// Device pointers of one context.  [2] arrays are ping-pong buffers indexed
// by the step parity a (read) / b = a ^ 1 (write).
struct DevState {
    int n;             // particles (slots)
    int ncol;          // colonies
    int ncols_total;   // columns over all colonies
    const DevGeom *geoms;
    const int *cbase;  // ncol + 1: first slot of each colony, then n (a compact copy for colony lookups)
    DevCounters *cnt;

    double *x[2], *y[2], *z[2];
    float4 *rel[2];    // FP32 offsets from the slot's bin corner (x, y, z) + radius (w)
    int *col[2];       // global column of the slot
    int *iz[2];        // z bin (grown-box coordinates, 1..nz)
    int *perm[2];      // slots sorted by (column, z bin, original index)
    int *colstart[2];  // ncols_total + 1 offsets into perm
    int *colcnt;       // per-column counter, zero between uses
    int *tmp;          // scatter scratch, n entries
    // column-sorted copies (optional: null skips them): srel[t] = rel[perm[t]],
    // siz[t] = iz[perm[t]], rank[perm[t]] = t; the sphere kernels walk these
    // contiguously instead of chasing perm
    float4 *srel[2];
    int *siz[2];
    int *rank[2];

    double *rad;
    int *orig;         // slot -> caller's index
    int8_t *ctype;     // cell_type

    double *vx, *vy, *vz, *wx, *wy, *wz;  // step outputs (slot order)
    float *vxf, *vyf, *vzf;               // velocity output of the FP32F sphere step

    // rod segments (null when the state holds spheres only)
    int has_rods;
    double *clen, *area, *bscale;
    double *theta[2], *phi[2];
    double4_32a *trig[2];  // (cos theta, sin theta, cos phi, sin phi)
    int *id, *cpu, *fuse_tip;
    int *tab[2];       // 13 planes: n_bnds, ids[4], cpus[4], sites[4]
    int *position, *fix_site, *fflag, *sflag, *nflag;
    int *dltd;         // 6 planes
    double *fc;        // 6 planes, force gather of the rod path
    float4 *axf;       // per segment, this step: FP32 axis (nx, ny, nz) and length (k_rod_book)
    double4_32a *mob;  // per segment: mobility (d0 + db, da - db, (d0 - db) / 2, 0) of its area,
                       // length and the viscosity (k_rod_mobility, on every state or parameter load)
    // FP32F rod pipeline (null until the first FP32F rod step): the gated pairs
    // of each segment in the reference's list order, kRodCap planes of n
    // entries (j, stencil code: bin offsets dx, dy, dz + 1 as a base-3 number in
    // bits 0-4, image shifts sx, sy + 1 in bits 5-8), written by k_rod_book
    int2 *rnb;
    int *rcnt;         // per segment: its gated pairs (may exceed kRodCap)
    double *rres;      // 6 x kRodCap planes of n: each pair's f1 + f2 (0-2), f1 - f2 (3-5)
    int2 *rwork;       // the pairs evaluated in FP64: (i, k | si << 8 | sj << 12)
    RodCtl *rctl;

    // FP32F neighbour list with a skin (null unless the context is in list mode)
    int *nbr;          // entries kNbrInline.. kNbrCap-1, one plane of n per entry: the
                       // neighbour slot (periodic images need no code: the fixed-point
                       // difference is the minimum image)
    int4 *lrec;        // per slot: x = list length (bits 0-7, saturating at 255) and the
                       // slot's place in its group's run of xlist (bits 8-17); y, z, w =
                       // the first kNbrInline entries
    // the entries past the inline ones, compacted for the step: per group of
    // 32 consecutive slots (one warp of k_list_step) the groups' entries lie
    // together, slot by slot in list order, from xoff[group] on
    int *xcnt;         // per group: its entries past the inline ones (then scanned into xoff)
    int *xoff;
    int *xlist;
    int4 *fxh[2];      // list path positions, ping-pong with x/y/z: high 32 bits of the
                       // 64-bit fixed-point x, y, z (FxGeom) and the FP32 radius bits --
                       // what a neighbour gathers
    unsigned *fxl[2];  // the low 32 bits, three planes of n (x, y, z)
    const FxGeom *fxg; // per colony
    int *pcap;         // null, or per slot 1 + kPairCap ints: the gated pairs of the last
                       // list step (count, then neighbour slots in accumulation order)
    unsigned long long *lkey;  // sort scratch, n (the load's sort and the list build): at each
                               // column position the counting sort gave a particle, its
                               // (z bin, caller index) key
    int *cellstart;    // ncells_total + 1 offsets of the cells in the sorted copies
    int ncells_total;
    int cols_max;      // largest column count of a colony
    ListCtl *lctl;
};

// Extension parameters of the differentiation form (k_adjoint.cu).
struct DiffParams {
    double gamma;        // two-body dashpot
    double mu;           // Stokes drag of spheres (0: mobility 1)
    const double *adh;   // per-slot adhesion energy (null: zero)
};

// ---- binning / counting sort (k_bin.cu) ----------------------------------
int launch_bin(const DevState &S, int b, int grid, int block, cudaStream_t st);
// gate (may be null): the kernels return at once when *gate == 0
int launch_scan(const int *in, int *out, int n, int *scratch, cudaStream_t st, const int *gate = nullptr);
size_t scan_scratch_ints(int n);
// ra: buffer whose FP32 offsets the sorted copies take (default b)
int launch_scatter_canon(const DevState &S, int b, int grid, int block, cudaStream_t st, int ra = -1,
                         const int *gate = nullptr);
int launch_rebuild(const DevState &S, int b, int *scan_scratch, int grid, int block, cudaStream_t st,
                   int ra = -1, const int *gate = nullptr);

// positions, radii, cell types, bins, offsets and identity column order of a
// freshly sorted state (buffer 0), gathered from the caller-order arrays
int launch_load_slots(const DevState &S, const double *ux, const double *uy, const double *uz, const double *ur,
                      const int *uct, const int *ucol, const int *uiz, const int *uperm, int grid, int block,
                      cudaStream_t st);
// *diff |= 1 when a given field (null: not compared) differs bit for bit from
// the device state of buffer a (slot s against caller index orig[s])
int launch_same_state(const DevState &S, int a, const double *x, const double *y, const double *z, const double *r,
                      const int *ct, unsigned long long *diff, int grid, int block, cudaStream_t st);
// state checks before a load: out[4] = {bad cell type, any FUNGI, largest radius bits, NaN radius}
int launch_check_state(const int *ct, const double *r, int n, unsigned long long *out, int grid, int block,
                       cudaStream_t st);

// caller-order staging -> slot order (set_state) and back (get_state)
int launch_user_bin(const DevState &S, const double *ux, const double *uy, const double *uz,
                     int *ucol, int *uiz, int grid, int block, cudaStream_t st);
// the caller's particles into column order: uperm[slot] = caller index (keys in lkey)
int launch_user_scatter_canon(const DevState &S, const int *ucol, const int *uiz, const int *colstart,
                               int *uperm, int grid, int block, cudaStream_t st);
int launch_gather_d(double *dst, const double *src, const int *perm, int n, int grid, int block, cudaStream_t st);
int launch_gather_i(int *dst, const int *src, const int *perm, int n, int planes, int grid, int block, cudaStream_t st);
int launch_scatter_d(double *dst, const double *src, const int *orig, int n, int grid, int block, cudaStream_t st);
int launch_scatter_f2d(double *dst, const float *src, const int *orig, int n, int grid, int block,
                       cudaStream_t st);
int launch_scatter_i(int *dst, const int *src, const int *orig, int n, int planes, int grid, int block, cudaStream_t st);
int launch_trig(const DevState &S, int b, int grid, int block, cudaStream_t st);

// neighbour-list export (k_bin.cu): mode 0 counts per caller index, mode 1 fills
int launch_pairs(const DevState &S, const DevParams &P, int a, int64_t *cnt_or_offs, int *idx,
                  int8_t *img, int mode, int grid, int block, cudaStream_t st);

// ---- spheres (k_sphere.cu) -----------------------------------------------
// force gather + wall + update + rebin of every slot, reading buffer a and
// writing buffer b; precision BMXG_FP64 / BMXG_FP32F
// resync (FP32F only): re-derive every slot's FP32 offsets and bin from its
// FP64 position this step
int launch_sphere_step(const DevState &S, const DevParams &P, double dt, int a, int precision,
                        int grid, int block, cudaStream_t st, int resync = 1);

// ---- FP32F neighbour list with a skin (k_list.cu) --------------------------
// decide: fold the last step's displacement into the bound and decide
// whether this step rebuilds; sets the graph conditional `cond` when use_cond
int launch_list_decide(const DevState &S, unsigned long long cond, int use_cond, cudaStream_t st);
// fixed-point positions of buffer a from its FP64 positions and radii (when the
// list starts on a state), and back (whenever the FP64 positions are read)
int launch_list_init(const DevState &S, int a, int grid, int block, cudaStream_t st);
int launch_list_to_fp64(const DevState &S, int a, int grid, int block, cudaStream_t st);
// axis ax (0 x, 1 y, 2 z) of it, also scattered to out in the caller's order (out[orig[i]])
int launch_list_to_fp64_axis(const DevState &S, int a, int ax, double *out, int block, cudaStream_t st);
// rebuild (gated on lctl->rebuild): bins of buffer a's positions into the
// list bins, column lists, and the list itself
// (returns the kernels it enqueues, kListBodyKernels)
int launch_list_rebuild(const DevState &S, const DevParams &P, int a, int *scan_scratch, int grid, int block,
                        int build_block, cudaStream_t st);
// the list build kernel alone (gated on lctl->rebuild), build_block threads per block
int launch_list_build(const DevState &S, const DevParams &P, int build_block, cudaStream_t st);
constexpr int kListBodyKernels = 12;
// force + wall + update over the list, reading buffer a and writing buffer b
// (grid = the SM count; passes of the block per chunk of slots, <= 0: a rule;
// persistent: one wave of blocks taking chunks from a counter, else one block
// per chunk)
int launch_list_step(const DevState &S, const DevParams &P, double dt, int a, int grid, int block, int passes,
                     cudaStream_t st, bool persistent = false);

// ---- one tile with the caller's ghosts (k_tile.cu) -------------------------
// The level's domain and the tile: cells are the domain's (1-based bins of
// the whole-domain step) offset by lo, the tile's first cell minus one, so
// that the tile's own cells are 1..nt and the one-cell halo 0 and nt + 1.
struct TileGeom {
    double plo[3], phi[3], len[3], dxi[3];
    int n[3], per[3];
    int lo[3], nt[3];
    int nbh_trivial;
};
// Device buffers of one tile call: positions, radii and cell types of the
// reals then the ghosts; the reals' outputs; cell scratch and counters.
struct TileBufs {
    double *x, *y, *z, *r;
    int *ct;
    double *ox, *oy, *oz, *vx, *vy, *vz;
    int *cell, *cnt, *start, *fill, *perm;
    unsigned long long *bad;  // [3]: a real outside the tile or a ghost outside the halo; a non-sphere;
                              // a non-finite new position
};
// bin, count, scan, scatter, order each cell by index, step the reals
int launch_tile_step(const TileBufs &B, const TileGeom &T, const DevParams &P, double dt, int nreal, int ntot,
                     int *scan_scratch, int nsm, cudaStream_t st);

// ---- rods and mixed states (k_rod.cu) ------------------------------------
int launch_rod_mobility(const DevState &S, const DevParams &P, int grid, int block, cudaStream_t st);
// list: also record each segment's gated pairs (the FP32F pipeline)
int launch_rod_book(const DevState &S, const DevParams &P, int a, bool list, int grid, int block, cudaStream_t st);
// the FP32F pipeline after the bookkeeping: FP32 pairs, FP64 pairs, per-segment sums
int launch_rod_pairs(const DevState &S, const DevParams &P, int a, int nsm, int n, cudaStream_t st);
int launch_rod_force(const DevState &S, const DevParams &P, int a, int precision, int grid, int block,
                      cudaStream_t st);
int launch_rod_update(const DevState &S, double dt, int a, int grid, int block, cudaStream_t st);
// one ParticleExchange substep: conc / out 3 planes (A, B, C), slot order; xpar host
int launch_exchange(const DevState &S, const DevParams &P, int a, const double *vol, const double *conc, double *out,
                    double dt, const double *xpar, int grid, int block, cudaStream_t st);
// start-up bond detection; counts[0] += bonds added, counts[1] += bonds past four
int launch_init_bonds(const DevState &S, const DevParams &P, int a, double rlim, unsigned long long *counts,
                      int grid, int block, cudaStream_t st);

// ---- differentiation form (k_adjoint.cu) ---------------------------------
int launch_dfwd(const DevState &S, const DevParams &P, const DiffParams &D, double dt, int a, int grid, int block,
                cudaStream_t st);
int launch_dadj(const DevState &S, const DevParams &P, const DiffParams &D, double dt, int a, const double *lin,
                double *lout, double *gacc, double *gadh, int grid, int block, cudaStream_t st);
int launch_dreduce(const double *gacc, int n, int planes, double *out, cudaStream_t st);

}  // namespace bmxg
