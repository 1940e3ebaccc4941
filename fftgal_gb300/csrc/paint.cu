// PCS (piecewise cubic spline) mass assignment for sm_103a.
//
// Restates the arithmetic of the reference's fft_p2g (src/fft.c:57-131):
// u = x * Ng/L - offset, base cell floor(u), fraction d = u - floor(u), the four
// cubic B-spline weights of src/fft.c:83-88, cells wrapped mod Ng.  The GPU
// organisation is new:
//
//  1. count   : every particle gets the key (tile, class) of its base cell.  The
//               grid is cut into tiles of at most 32 x 16 x 32 cells (i, j, k;
//               FP32 grids with Ng >= 64) or 16 x 16 x 32 (FP64, smaller Ng);
//               per axis the class says whether the particle's stencil (over
//               all painted grids) reaches into the lower (1) or upper (2)
//               neighbour tile, or neither (0).  Only the key histogram is
//               written (fire-and-forget atomics).
//  2. scan    : exclusive prefix sum of the key histogram, copied to a cursor
//               array.
//  3. scatter : the key is formed again and each particle's record is written
//               at the slot its key's cursor atomic returns.  The order within
//               a key depends on the atomics' order; the FP32 paint sums in
//               fixed point, so the painted grid does not.
//  4. paint   : one CTA per tile owns its cells.  It pulls the particles of its
//               own tile and only the boundary classes of its 26 neighbours,
//               accumulates their weights in shared memory and writes every
//               owned cell exactly once (no global atomics, no zeroing pass).
//
// FP32 grids (paint_coop_kernel, persistent over tiles): each lane prepares
// one particle (cell indices and the 3 x 4 weights of one grid) in shared
// memory, then the warp deposits the particles one at a time with lane =
// (grid, i row, j row), each lane adding its 4 k cells; the shared layout makes
// every such step touch 32 distinct banks.  One grid of 32-row tiles, or two
// of 16-row tiles, take 79 KB of sums: two 512-thread CTAs per SM.  The two
// interlacing grids of 32-row tiles are painted by separate CTAs, one grid
// each, from one sort.  Sums are 32-bit fixed point with a
// per-tile scale 2^-s, s the largest value for which no cell can exceed 2^32 (a
// particle adds at most (2/3)^3 of its weight to a cell): the tile's particle
// total bounds every cell, and only where that bound leaves fewer than 21
// fraction bits does a first pass count particles per 4^3-cell block.  A tile
// whose bound still leaves fewer than 16 bits (a dense clump: more than about
// 2e5 particles near one cell) paints one grid at a time into 64-bit sums
// with 22 fraction bits over the same shared memory, since at 12-15 bits the
// many tiny products at a stencil's edge round to zero and bias the edge cells
// low by several percent.  Integer sums are order independent, so the painted
// grid is bit-reproducible run to run.
// FP64 grids (paint_tile_f64_kernel) reproduce the reference's FP64 weight
// arithmetic op for op and accumulate in FP64, one thread per particle.
#include "internal.h"
#include "common.cuh"

#include <math.h>
#include <string.h>
#include <vector>

namespace fg {

constexpr int kTileExt[3] = {16, 16, 32};    // i, j, k
constexpr int kTileExt1[3] = {32, 16, 32};   // FP32 paints of one grid (Ng >= 64)
constexpr int kMaxPaintGrids = 2;
// dense tiles (fewer 32-bit fraction bits than kWideBelow): 64-bit sums with
// kWideBits fraction bits, one grid per pass.  At 16-19 bits the 32-bit sums
// round the tiny products at a dense clump's stencil edge by up to 1.4 % of
// those cells' values (1e-6 of the clump's peak cell, 1e-5 of its mass); the
// clustered 1e8-galaxy lognormal mock has many such tiles, whose tile paint
// the 64-bit passes took from 13.0 to 15.8 ms (Ng = 1024) at a threshold of 20
constexpr int kWideBelow = 16;
constexpr int kWideBits = 22;
// FP32 shared layout: cell (li, lj, lk) of grid g at g*kGS + li*kSI + lj*kSJ +
// kPadK + lk.  kSI = 8 and kSJ = 6 (mod 32) put the 16 rows (li+a, lj+b), a, b
// < 4, of one stencil in 16 distinct banks of one parity, and the odd kGS gives
// the other grid the other parity: with each lane of the second grid taking
// its 4 k cells in the order s ^ ((b1 - b0) & 1) (its stencil is shifted by
// b1 - b0 cells along k), every one of the 4 atomic steps of a particle touches
// 32 distinct banks.  kPadK columns on either side of a row take the stencil
// cells beyond the tile along k, so a particle's 4 k cells are always
// contiguous; stencil rows outside the tile in i or j (local index kOut) are
// skipped.
constexpr int kPadK = 3;
constexpr int kSJ = 38, kSI = 616, kGS = 9849;
constexpr uint32_t kOut = 255u;
static_assert(15 * kSI + 15 * kSJ + kSJ <= kGS, "tile does not fit the layout");
static_assert(32 + 2 * kPadK <= kSJ, "row padding");
static_assert(kSI % 32 == 8 && kSJ % 32 == 6 && kGS % 2 == 1, "bank layout");
// the accumulators: two grids of 16 i rows, or one grid of 32 i rows (row li
// at li * kSI)
constexpr int kAccWords = 2 * kGS > 32 * kSI ? 2 * kGS : 32 * kSI;
static_assert(31 * kSI + 15 * kSJ + kSJ <= kAccWords, "32-row tile does not fit the layout");
constexpr size_t kAccBytes = (sizeof(uint32_t) * kAccWords + 15) / 16 * 16;
// The tile-paint CTA: 512 threads, two CTAs per SM, the two grids of 16 i
// rows at stride kGS or one grid of 32 rows.  (One 1024-thread CTA per SM
// holding both grids of 32-row tiles, 158 KB of sums, was measured slower than
// two one-grid CTAs per SM.)  A dense tile's 64-bit sums hold 16 i rows.
constexpr int kWideRows = kAccWords / 2 / kSI;
static_assert(kWideRows == 16, "64-bit rows");
// largest fixed-point scale: products stay below 2^22 so the FMA trick of
// deposit4 converts them to integers exactly
constexpr int kMaxFixBits = 23;
// the per-block count that can raise a dense tile's scale runs only when its
// particle total leaves fewer bits than this (tiles of more than about 6900
// particles): at >= 21 fraction bits a deposit rounds by at most 2^-22 of a
// unit weight, inside FP32 grid accuracy even where the deconvolution
// amplifies the noise of the corner bins, so the extra pass over the tile's
// records (most of 1 ms of the tile paint for a 1e8-galaxy lognormal mock at
// Ng=1024) is skipped for moderately dense tiles
constexpr int kBlockCountBelow = 21;
// FP64 shared layout: dense [16][16][32]
constexpr int kT3 = 16 * 16 * 32;
// per-tile block counts: 4^3-cell blocks over the tile plus a 4-cell margin
constexpr int kBlk = 4;
__host__ __device__ constexpr int blk_dim(int a) { return a == 1 ? (16 + 8) / kBlk : (32 + 8) / kBlk; }  // 10, 6, 10
constexpr int kBlkN = blk_dim(0) * blk_dim(1) * blk_dim(2);

struct AxisParams {
    // FP32 path: x * h - o as double-float (h = Ng/L, o = offset of grid g)
    float h_hi, h_lo;
    float o_hi[kMaxPaintGrids], o_lo[kMaxPaintGrids];
    // FP32 path: u_g = u_0 + delta_g, delta_g = o_0 - o_g in units of 2^-fb
    int dq[kMaxPaintGrids];
    // FP64 path
    double h;
    double o[kMaxPaintGrids];
};

struct PaintParams {
    AxisParams ax[3];
    // FP32 redshift-space displacement (v[0] null: none)
    const float *v[3];
    float los[3], aHinv;
    int Ng, Ng_pad, ngrids;
    int fb;                  // FP32 path: fraction bits of the packed cell coordinate
    int nt[3];
    const int *tile_of[3];   // [Ng] per axis
    int tshift[3];           // log2 of the tile extent when every tile of the axis has it, else -1
    const int *start[3];     // [nt + 1] per axis
};

// ---- redshift-space displacement ---------------------------------------------
// x + ((los . v) / aH) los, the operation order of src/gal.c:69-72 in FP32 with
// explicit FMAs, so the key and scatter kernels displace a particle identically
__device__ __forceinline__ void rsd_displace(const PaintParams &pp, long p, float pos[3]) {
    if (!pp.v[0]) return;
    const float vd = fmaf(pp.los[2], pp.v[2][p], fmaf(pp.los[1], pp.v[1][p], pp.los[0] * pp.v[0][p]));
    const float s = pp.aHinv * vd;
#pragma unroll
    for (int a = 0; a < 3; ++a) pos[a] = fmaf(s, pp.los[a], pos[a]);
}
__device__ __forceinline__ void rsd_displace(const PaintParams &, long, double *) {}

// ---- per-axis cell coordinate ----------------------------------------------

__device__ __forceinline__ void coord(float x, const AxisParams &a, int g, int Ng, int &b, float &d) {
    // u = x*h - o with the rounding errors of the product and the subtraction
    // carried in a second float, then split into floor and fraction
    const float p = x * a.h_hi;
    const float pe = fmaf(x, a.h_hi, -p) + x * a.h_lo;
    const float s = p - a.o_hi[g];
    const float bv = s - p;
    const float se = (p - (s - bv)) + (-a.o_hi[g] - bv);
    const float lo = (pe + se) - a.o_lo[g];
    const float fb = floorf(s);
    float fr = (s - fb) + lo;
    int ib = (int)fb;
    if (fr < 0.f) {
        fr += 1.f;
        ib -= 1;
    } else if (fr >= 1.f) {
        fr -= 1.f;
        ib += 1;
    }
    ib %= Ng;
    if (ib < 0) ib += Ng;
    b = ib;
    d = fr;
}

__device__ __forceinline__ void coord(double x, const AxisParams &a, int g, int Ng, int &b, double &d) {
    // src/fft.c:68-82, evaluated without contraction so it rounds like the host
    const double u = __dsub_rn(__dmul_rn(x, a.h), a.o[g]);
    const int g1 = (int)floor(u);
    d = __dsub_rn(u, (double)g1);
    b = (g1 % Ng + Ng) % Ng;
}

__device__ __forceinline__ void pcs_weights(float d, float w[4]) {
    const float e = 1.f - d;
    const float d2 = d * d;
    w[0] = e * e * e * (1.f / 6.f);
    w[1] = ((3.f * d - 6.f) * d2 + 4.f) * (1.f / 6.f);
    w[2] = (((-3.f * d + 3.f) * d + 3.f) * d + 1.f) * (1.f / 6.f);
    w[3] = d2 * d * (1.f / 6.f);
}

__device__ __forceinline__ void pcs_weights(double d, double w[4]) {
    // src/fft.c:83-88 in the reference's operation order, no FMA contraction
    const double e = __dsub_rn(1.0, d);
    const double d2 = __dmul_rn(d, d);
    w[0] = __ddiv_rn(__dmul_rn(__dmul_rn(e, e), e), 6.0);
    w[1] = __ddiv_rn(__dadd_rn(__dmul_rn(__dsub_rn(__dmul_rn(3.0, d), 6.0), d2), 4.0), 6.0);
    w[2] = __ddiv_rn(
        __dadd_rn(__dmul_rn(__dadd_rn(__dmul_rn(__dadd_rn(__dmul_rn(-3.0, d), 3.0), d), 3.0), d), 1.0),
        6.0);
    w[3] = __ddiv_rn(__dmul_rn(d2, d), 6.0);
}

// FP32 path: the grid-0 base cell b0 and the fraction as fb-bit fixed point;
// every other grid's cell is derived from these with an exact integer shift,
// identically in the key and the paint kernels.
__device__ __forceinline__ void cell0(float x, const AxisParams &a, int Ng, int fb, int &b0, uint32_t &dq) {
    float d;
    coord(x, a, 0, Ng, b0, d);
    const uint32_t one = 1u << fb;
    dq = (uint32_t)(d * (float)one);
    dq = dq >= one ? one - 1 : dq;
}

__device__ __forceinline__ void cell_g(int b0, uint32_t dq, int delta, int fb, int Ng, int &bg, uint32_t &dgq) {
    const int t = (int)dq + delta;  // |delta| <= 2^fb
    dgq = (uint32_t)t & ((1u << fb) - 1);
    bg = b0 + (t >> fb);            // arithmetic shift: floor division
    bg += bg < 0 ? Ng : 0;
    bg -= bg >= Ng ? Ng : 0;
}

// local index of stencil cell s (0..3) of base cell b: (b - 1 + s) mod Ng
// relative to the tile start t0, or -1 outside [0, te)
__device__ __forceinline__ int local_cell(int b, int s, int Ng, int t0, int te) {
    int c = b - 1 + s;
    c = c < 0 ? c + Ng : (c >= Ng ? c - Ng : c);
    const int l = c - t0;
    return (l >= 0 && l < te) ? l : -1;
}

template <typename P> struct Rec;
template <> struct Rec<float> { using type = uint4; };  // per axis (b0 << fb) | fraction
template <> struct Rec<double> { struct type { double x, y, z; }; };

// ---- 1. key + histogram -------------------------------------------------------

// the key of a particle; for FP32 positions also its packed record words
// (b0 << fb) | fraction per axis
template <typename P>
__device__ __forceinline__ uint32_t paint_key_of(const P pos[3], const PaintParams &pp, uint32_t *rec = nullptr) {
    const int Ng = pp.Ng;
    int t[3], cls[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        int b0;
        uint32_t dq0 = 0;
        if constexpr (sizeof(P) == 4) {
            cell0(pos[a], pp.ax[a], Ng, pp.fb, b0, dq0);
            if (rec) rec[a] = ((uint32_t)b0 << pp.fb) | dq0;
        } else {
            P d;
            coord(pos[a], pp.ax[a], 0, Ng, b0, d);
        }
        int ta, t0, te;
        if (pp.tshift[a] >= 0) {
            ta = b0 >> pp.tshift[a];
            t0 = ta << pp.tshift[a];
            te = 1 << pp.tshift[a];
        } else {
            ta = pp.tile_of[a][b0];
            t0 = pp.start[a][ta];
            te = pp.start[a][ta + 1] - t0;
        }
        int rmin = b0 - t0, rmax = b0 - t0;
        for (int g = 1; g < pp.ngrids; ++g) {
            int bg;
            if constexpr (sizeof(P) == 4) {
                uint32_t dgq;
                cell_g(b0, dq0, pp.ax[a].dq[g], pp.fb, Ng, bg, dgq);
            } else {
                P dg;
                coord(pos[a], pp.ax[a], g, Ng, bg, dg);
            }
            int dl = bg - b0;  // -1, 0 or +1 after undoing a wrap
            dl -= dl > 1 ? Ng : 0;
            dl += dl < -1 ? Ng : 0;
            rmin = min(rmin, b0 - t0 + dl);
            rmax = max(rmax, b0 - t0 + dl);
        }
        t[a] = ta;
        cls[a] = pp.nt[a] == 1 ? 0 : (rmin - 1 < 0 ? 1 : (rmax + 2 >= te ? 2 : 0));
    }
    return (uint32_t)((((long)t[0] * pp.nt[1] + t[1]) * pp.nt[2] + t[2]) * 27 + cls[0] * 9 + cls[1] * 3 + cls[2]);
}

template <typename P>
__global__ void paint_key_kernel(const P *__restrict__ x, const P *__restrict__ y,
                                 const P *__restrict__ z, long Np, PaintParams pp,
                                 uint32_t *__restrict__ hist, const DevScalars *__restrict__ ds) {
    if (ds) Np = ds->Np;
    for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < Np; p += (long)gridDim.x * blockDim.x) {
        P pos[3] = {x[p], y[p], z[p]};
        rsd_displace(pp, p, pos);
        atomicAdd(&hist[paint_key_of<P>(pos, pp)], 1u);
    }
}

// ---- 2. exclusive scan of the histogram (in place, n + 1 entries) ------------------

constexpr int kScanThreads = 1024;
constexpr int kScanPer = 4;
constexpr int kScanBlock = kScanThreads * kScanPer;

__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t *warp_sums, uint32_t *total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t u = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += u;
    }
    if (lane == 31) warp_sums[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
        uint32_t ws = lane < nw ? warp_sums[lane] : 0;
        uint32_t wi = ws;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t u = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += u;
        }
        if (lane < nw) warp_sums[lane] = wi - ws;
        if (lane == 31) *total = wi;
    }
    __syncthreads();
    const uint32_t r = warp_sums[wid] + inc - v;
    __syncthreads();
    return r;
}

__global__ void scan_block_sums(const uint32_t *__restrict__ a, long n, uint32_t *__restrict__ bsum) {
    __shared__ uint32_t ws[32];
    __shared__ uint32_t tot;
    const long base = (long)blockIdx.x * kScanBlock + threadIdx.x * kScanPer;
    uint32_t s = 0;
#pragma unroll
    for (int i = 0; i < kScanPer; ++i)
        if (base + i < n) s += a[base + i];
    block_exclusive_scan(s, ws, &tot);
    if (threadIdx.x == 0) bsum[blockIdx.x] = tot;
}

__global__ void scan_top(uint32_t *bsum, long nb) {
    __shared__ uint32_t ws[32];
    __shared__ uint32_t tot;
    uint32_t carry = 0;
    for (long c0 = 0; c0 < nb; c0 += blockDim.x) {
        const long i = c0 + threadIdx.x;
        const uint32_t v = i < nb ? bsum[i] : 0;
        const uint32_t e = block_exclusive_scan(v, ws, &tot);
        if (i < nb) bsum[i] = carry + e;
        carry += tot;
        __syncthreads();
    }
}

__global__ void scan_apply(uint32_t *__restrict__ a, long n, const uint32_t *__restrict__ bsum) {
    __shared__ uint32_t ws[32];
    __shared__ uint32_t tot;
    const long base = (long)blockIdx.x * kScanBlock + threadIdx.x * kScanPer;
    uint32_t v[kScanPer];
    uint32_t s = 0;
#pragma unroll
    for (int i = 0; i < kScanPer; ++i) {
        v[i] = base + i < n ? a[base + i] : 0;
        s += v[i];
    }
    uint32_t e = block_exclusive_scan(s, ws, &tot) + bsum[blockIdx.x];
#pragma unroll
    for (int i = 0; i < kScanPer; ++i) {
        if (base + i < n) a[base + i] = e;
        e += v[i];
    }
}

static int exclusive_scan(uint32_t *a, long n, uint32_t *bsum, cudaStream_t st) {
    const long nb = ceil_div(n, kScanBlock);
    scan_block_sums<<<(unsigned)nb, kScanThreads, 0, st>>>(a, n, bsum);
    scan_top<<<1, kScanThreads, 0, st>>>(bsum, nb);
    scan_apply<<<(unsigned)nb, kScanThreads, 0, st>>>(a, n, bsum);
    FG_LAUNCHED(3);
    return OK;
}

// ---- 3. scatter into key order ------------------------------------------------------

template <typename P>
__global__ void paint_scatter_kernel(const P *__restrict__ x, const P *__restrict__ y,
                                     const P *__restrict__ z, long Np, PaintParams pp,
                                     uint32_t *__restrict__ cursor,
                                     typename Rec<P>::type *__restrict__ sorted,
                                     const DevScalars *__restrict__ ds) {
    if (ds) Np = ds->Np;
    for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < Np; p += (long)gridDim.x * blockDim.x) {
        P pos[3] = {x[p], y[p], z[p]};
        rsd_displace(pp, p, pos);
        typename Rec<P>::type r;
        uint32_t k;
        if constexpr (sizeof(P) == 4) {
            uint32_t w[3];
            k = paint_key_of<P>(pos, pp, w);
            r = make_uint4(w[0], w[1], w[2], 0u);
        } else {
            k = paint_key_of<P>(pos, pp);
            r.x = pos[0];
            r.y = pos[1];
            r.z = pos[2];
        }
        sorted[atomicAdd(&cursor[k], 1u)] = r;
    }
}

// ---- 4. tile paint ---------------------------------------------------------------------

constexpr int kPaintThreads = 512;
constexpr int kStageParts = 16;  // particles staged per warp and round
constexpr int kMaxSeg = 125;

struct PaintOut {
    void *out[kMaxPaintGrids];
    double scale[kMaxPaintGrids];
    int accumulate[kMaxPaintGrids];
    const DevScalars *ds;  // if set, the scales are ds->scale
};

// Tile geometry and the flattened list of particle segments a tile pulls:
// its own key range for every class and the boundary classes of the (up to
// 26, deduplicated for 1 or 2 tiles per axis) neighbours.
struct TileSegs {
    int t0[3], te[3];
    int nseg;
    uint32_t total;
};

__device__ void tile_geometry(const PaintParams &pp, unsigned tile, TileSegs &ts) {
    const int nt1 = pp.nt[1], nt2 = pp.nt[2];
    const int tt[3] = {(int)(tile / (nt1 * nt2)), (int)((tile / nt2) % nt1), (int)(tile % nt2)};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        ts.t0[a] = pp.start[a][tt[a]];
        ts.te[a] = pp.start[a][tt[a] + 1] - ts.t0[a];
    }
}

// thread q's segment of `tile` (q < the returned count): first sorted index b
// and length cnt.  Issued a tile ahead so the loads overlap the write-out.
__device__ int tile_segment(const PaintParams &pp, const uint32_t *__restrict__ off, unsigned tile, int q,
                            uint32_t &b, uint32_t &cnt) {
    const int nt1 = pp.nt[1], nt2 = pp.nt[2];
    const int tt[3] = {(int)(tile / (nt1 * nt2)), (int)((tile / nt2) % nt1), (int)(tile % nt2)};
    // per axis the options (tile, class): the own tile with every class, then
    // the lower neighbour's particles reaching up (class 2) and the upper
    // neighbour's reaching down (class 1); both from the same tile when nt = 2
    int nopt[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) nopt[a] = pp.nt[a] == 1 ? 1 : 5;
    const int ncomb = nopt[0] * nopt[1] * nopt[2];  // <= 125
    b = 0;
    cnt = 0;
    if (q < ncomb) {
        const int idx[3] = {q / (nopt[1] * nopt[2]), (q / nopt[2]) % nopt[1], q % nopt[2]};
        int ot[3], oc[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const int nt = pp.nt[a], x = idx[a];
            if (x < 3) {
                ot[a] = tt[a];
                oc[a] = nt == 1 ? 0 : x;
            } else {
                const int lo = (tt[a] + nt - 1) % nt, hi = (tt[a] + 1) % nt;
                if (nt == 2) {
                    ot[a] = hi;
                    oc[a] = x == 3 ? 1 : 2;
                } else {
                    ot[a] = x == 3 ? lo : hi;
                    oc[a] = x == 3 ? 2 : 1;
                }
            }
        }
        const long key = (((long)ot[0] * nt1 + ot[1]) * nt2 + ot[2]) * 27 + oc[0] * 9 + oc[1] * 3 + oc[2];
        b = off[key];
        cnt = off[key + 1] - b;
    }
    return ncomb;
}

// publish the fetched segments in shared memory (every thread takes part)
__device__ void tile_publish(int ncomb, uint32_t b, uint32_t cnt, uint32_t *seg_begin, uint32_t *seg_pref,
                             uint32_t *scan_ws, TileSegs &ts) {
    const int q = threadIdx.x;
    const uint32_t pref = block_exclusive_scan(cnt, scan_ws, &scan_ws[32]);  // scan_ws[33]
    const uint32_t tot = scan_ws[32];
    if (q < ncomb) {
        seg_begin[q] = b;
        seg_pref[q] = pref;
    }
    if (q == 0) seg_pref[ncomb] = tot;
    __syncthreads();
    ts.nseg = ncomb;
    ts.total = tot;
}

__device__ void tile_segments(const PaintParams &pp, const uint32_t *__restrict__ off, uint32_t *seg_begin,
                              uint32_t *seg_pref, uint32_t *scan_ws, TileSegs &ts) {
    tile_geometry(pp, blockIdx.x, ts);
    uint32_t b, cnt;
    const int ncomb = tile_segment(pp, off, blockIdx.x, threadIdx.x, b, cnt);
    tile_publish(ncomb, b, cnt, seg_begin, seg_pref, scan_ws, ts);
}

// index of particle q of the flattened segment list (largest segment whose
// prefix is <= q; empty segments are skipped automatically)
__device__ __forceinline__ uint32_t seg_index(uint32_t q, const uint32_t *seg_begin, const uint32_t *seg_pref,
                                              int nseg) {
    int lo = 0, hi = nseg - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (seg_pref[mid] <= q) lo = mid;
        else hi = mid - 1;
    }
    return seg_begin[lo] + (q - seg_pref[lo]);
}

// per warp: the staged particles of one round, slot = particle + 16 * grid
struct __align__(16) StageBuf {
    uint4 loc[32];     // per axis: 4 packed local cell indices (255 = outside the tile); .w unused
    float4 w[3][32];   // per axis: PCS weights (k weights pre-scaled by 2^s)
};

__device__ __forceinline__ uint32_t pack_local(int b, int Ng, int t0, int te, uint32_t outv) {
    uint32_t r = 0;
#pragma unroll
    for (int s = 0; s < 4; ++s) {
        int cs = b - 1 + s;  // in [-1, Ng + 2): one correction each way (Ng >= 2)
        cs += cs < 0 ? Ng : 0;
        cs -= cs >= Ng ? Ng : 0;
        const int l = cs - t0;
        r |= ((unsigned)l < (unsigned)te ? (uint32_t)l : outv) << (8 * s);
    }
    return r;
}

// deposit staged particles: lane = (grid, i row, j row), or (particle parity,
// i row, j row) when one grid is painted; every lane adds its row's 4 k
// cells.  By the bank layout each of the 4 atomic steps is a single
// shared-memory wavefront (two grids).  The loop is unrolled so that the
// shared loads of the next particles overlap the atomics of the current one
// (unrolled by 4: 2 % faster than by 2 at Ng = 1024).  One grid: 32
// particles staged per round by all lanes and the half warps depositing
// alternate ones took the one-grid tile paint from 11.7 to 6.9 ms at Ng=1024
// (with the grid count a template parameter of the kernel, which also took
// the two-grid paint from 12.4 to 11.9 ms).
// Stencil cells outside the tile (local index kOut) are skipped.
// slot of particle p of grid g in the stage buffer: the two grids' records
// interleave so that lanes reading both fall in different banks
__device__ __forceinline__ int stage_slot(int p, int g) { return 2 * p + g; }

// add round(w * wz) to the cell at offset `off`: 32-bit sums, or 64-bit sums
// (WIDE, offsets counted in 64-bit cells); w * wz < 2^22
template <bool WIDE>
__device__ __forceinline__ void dep_one(uint32_t *acc, int off, float w, float wz) {
    const float M = 12582912.0f;  // 1.5 * 2^23: FMA onto it rounds w * wz to an integer
    const uint32_t q = __float_as_uint(fmaf(w, wz, M)) - 0x4B400000u;
    if (WIDE)
        atomicAdd(reinterpret_cast<unsigned long long *>(acc) + off, (unsigned long long)q);
    else
        atomicAdd(acc + off, q);
}

// One particle of grid g for lane (a, b).
// FAST (no tile spans a periodic axis): loc.x / loc.y are the offsets of the
// particle's cells s ^ par for s = 0 and 1 in the stencil row (a, b) = (0, 0),
// relative to the accumulator, with par the cell-order bit; row (a, b) adds
// a*kSI + b*kSJ (lane_off).  loc.z has bit 4a + b set for the rows inside the
// tile.  The 4 k cells are contiguous (kPadK columns take those beyond the tile).
// Otherwise loc.x / loc.y hold the 4 local i / j indices as bytes (kOut outside
// the tile) and loc.z the 4 padded k cells as bytes, in step order.
// The k weights are stored in step order.
template <bool WIDE, bool FAST>
__device__ __forceinline__ void deposit_one(uint32_t *acc, const StageBuf &sb, int slot, int g, int a, int b,
                                            int lane_off) {
    const uint4 loc = sb.loc[slot];
    const float w = reinterpret_cast<const float *>(&sb.w[0][slot])[a] *
                    reinterpret_cast<const float *>(&sb.w[1][slot])[b];
    const float4 wz = sb.w[2][slot];
    if (FAST) {
        if (!((loc.z >> (4 * a + b)) & 1u)) return;  // a stencil row outside the tile
        const int o0 = (int)loc.x + lane_off, o1 = (int)loc.y + lane_off;
        dep_one<WIDE>(acc, o0, w, wz.x);
        dep_one<WIDE>(acc, o1, w, wz.y);
        dep_one<WIDE>(acc, o0 + 2, w, wz.z);
        dep_one<WIDE>(acc, o1 + 2, w, wz.w);
    } else {
        const uint32_t li = (loc.x >> (8 * a)) & 255u;
        const uint32_t lj = (loc.y >> (8 * b)) & 255u;
        if ((li | lj) >= 32u) return;  // kOut: a stencil row outside the tile
        const int row = g * kGS + (int)(li * kSI + lj * kSJ);
        dep_one<WIDE>(acc, row + (int)(loc.z & 255u), w, wz.x);
        dep_one<WIDE>(acc, row + (int)((loc.z >> 8) & 255u), w, wz.y);
        dep_one<WIDE>(acc, row + (int)((loc.z >> 16) & 255u), w, wz.z);
        dep_one<WIDE>(acc, row + (int)(loc.z >> 24), w, wz.w);
    }
}

template <bool WIDE, bool FAST>
__device__ __forceinline__ void deposit_all(uint32_t *acc, const StageBuf &sb, int np, int ngr, int lane) {
    const int h = lane >> 4, a = (lane >> 2) & 3, b = lane & 3;
    const int lane_off = a * kSI + b * kSJ;
    if (ngr > 1) {
#pragma unroll 4
        for (int p = 0; p < np; ++p) deposit_one<WIDE, FAST>(acc, sb, stage_slot(p, h), h, a, b, lane_off);
    } else {
        // one grid: 32 particles staged in slots 0..31, the half warps
        // deposit alternate ones; unrolled fully, so that the shared loads of
        // later particles are issued among the atomics of earlier ones (10.65
        // ms against 10.87 by 8, 11.18 by 4, 11.45 by 2 and 11.97 by 1, both
        // grids at Ng = 1024)
#pragma unroll 16
        for (int p = h; p < np; p += 2) deposit_one<WIDE, FAST>(acc, sb, p, 0, a, b, lane_off);
    }
}

// largest fixed-point exponent s for which `n` contributors to one cell cannot
// overflow its 32-bit sum: each adds round(w 2^s) <= 8/27 2^s + 1/2 (the
// largest PCS weight product is (2/3)^3), so n (16 2^s + 27) < 54 2^32 is
// required.  Exact integer arithmetic; a result below kWideBelow selects the
// 64-bit sums.
__device__ __forceinline__ int fix_bits_for(uint32_t n) {
    if (n == 0) return kMaxFixBits;
    const unsigned long long x = (54ull << 32) / n;
    if (x <= 28) return -1;
    const unsigned long long q = (x - 28) >> 4;
    const int fb = q == 0 ? -1 : 63 - __clzll((long long)q);
    return fb > kMaxFixBits ? kMaxFixBits : fb;
}

// Pass B over the tile's records: each warp stages 16 particles for both
// grids (NGS = 2: lanes 0..15 grid 0, 16..31 grid 1) or 32 particles of grid
// g1 (NGS = 1), then deposits them, into 32-bit sums or (WIDE) the 64-bit sums
// of grid g1; the records of the warp's next batch are loaded before the
// deposit so their latency hides behind it
template <int NGS, bool WIDE>
__device__ __forceinline__ void paint_records(uint32_t *acc, StageBuf &sb, const uint4 *__restrict__ sorted,
                                              const uint32_t *seg_begin, const uint32_t *seg_pref,
                                              const TileSegs &ts, const PaintParams &pp, const bool *cyc,
                                              bool fast, float fscale, int g1, const uint32_t (*loctab)[40],
                                              const uint32_t (*masktab)[40], int lane, int warp) {
    const int Ng = pp.Ng, fb = pp.fb, nseg = ts.nseg;
    const uint32_t total = ts.total;
    constexpr int nwarp = kPaintThreads / 32;
    const int parts = NGS > 1 ? kStageParts : 2 * kStageParts;  // particles per warp and round
    const int gs = NGS > 1 ? lane / kStageParts : g1;             // the grid this lane stages
    const int gofs = (WIDE || NGS == 1) ? 0 : gs * kGS;           // and its accumulator
    const float inv = __int_as_float((127 - fb) << 23);            // 2^-fb (fb <= 24)
    const uint32_t bstride = (uint32_t)nwarp * parts;
    uint32_t base = (uint32_t)warp * parts;
    uint4 rec = make_uint4(0, 0, 0, 0);
    {
        const uint32_t q = base + (lane & (parts - 1));
        if (q < total) rec = sorted[seg_index(q, seg_begin, seg_pref, nseg)];
    }
    for (; base < total; base += bstride) {
        const uint32_t q = base + (lane & (parts - 1));
        const bool valid = q < total;
        const int slot = NGS > 1 ? stage_slot(lane & (kStageParts - 1), gs) : lane;
        int bgv[3] = {0, 0, 0}, lv[3] = {0, 0, 0};
        uint32_t par = 0;
        float4 wk = make_float4(0.f, 0.f, 0.f, 0.f);
        if (valid) {
            const uint32_t rw[3] = {rec.x, rec.y, rec.z};
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                const int b0 = (int)(rw[a] >> fb);
                int bg;
                uint32_t dgq;
                cell_g(b0, rw[a] & ((1u << fb) - 1), pp.ax[a].dq[gs], fb, Ng, bg, dgq);
                float w[4];
                pcs_weights((float)dgq * inv, w);
                if (a == 2) {
                    wk = make_float4(w[0] * fscale, w[1] * fscale, w[2] * fscale, w[3] * fscale);
                    par = (uint32_t)(bg - b0) & 1u;
                } else {
                    sb.w[a][slot] = make_float4(w[0], w[1], w[2], w[3]);
                }
                // local index of the first stencil cell (periodic images
                // folded to the nearest copy of the tile)
                int l = bg - 1 - ts.t0[a];
                l -= l > Ng / 2 ? Ng : 0;
                l += l < -Ng / 2 ? Ng : 0;
                bgv[a] = bg;
                lv[a] = l;
            }
        }
        if (NGS == 1) {
            // one grid: the half warps deposit particles 2m and 2m + 1 together.
            // A first cell's bank parity is that of lv[2] + kPadK (the row
            // offsets kSI, kSJ are even), so particle 2m + 1 takes its k cells in
            // the order s ^ par that puts the pair's cells of every step in banks
            // of opposite parity, 16 distinct banks each: one wavefront per step
            const int other = __shfl_xor_sync(0xffffffffu, lv[2], 1);
            par = (lane & 1) ? (uint32_t)(((lv[2] ^ other) & 1) ^ 1) : 0u;
        }
        if (valid) {
            if (par) wk = make_float4(wk.y, wk.x, wk.w, wk.z);  // k cells in the order s ^ 1
            sb.w[2][slot] = wk;
            const bool kmiss = !cyc[2] && (lv[2] < -3 || lv[2] >= ts.te[2]);  // stencil misses the tile
            uint4 loc;
            if (fast) {
                const uint32_t mi = (unsigned)(lv[0] + 4) < 40u ? masktab[0][lv[0] + 4] : 0u;
                const uint32_t mj = (unsigned)(lv[1] + 4) < 40u ? masktab[1][lv[1] + 4] : 0u;
                const int b0 = gofs + lv[0] * kSI + lv[1] * kSJ + lv[2] + kPadK + (int)par;
                loc = make_uint4((uint32_t)b0, (uint32_t)(b0 + 1 - 2 * (int)par), kmiss ? 0u : mi * mj, 0u);
            } else {
                uint32_t li, lj, lk;
                li = cyc[0] ? pack_local(bgv[0], Ng, ts.t0[0], ts.te[0], kOut)
                            : ((unsigned)(lv[0] + 4) < 40u ? loctab[0][lv[0] + 4] : 0xFFFFFFFFu);
                lj = cyc[1] ? pack_local(bgv[1], Ng, ts.t0[1], ts.te[1], kOut)
                            : ((unsigned)(lv[1] + 4) < 40u ? loctab[1][lv[1] + 4] : 0xFFFFFFFFu);
                if (cyc[2])
                    lk = pack_local(bgv[2], Ng, ts.t0[2], ts.te[2], 0u) + 0x01010101u * kPadK;
                else
                    lk = (uint32_t)(kmiss ? 0 : lv[2] + kPadK) * 0x01010101u + 0x03020100u;
                if (par) lk = ((lk & 0x00FF00FFu) << 8) | ((lk >> 8) & 0x00FF00FFu);
                loc = make_uint4(kmiss ? 0xFFFFFFFFu : li, lj, lk, 0u);
            }
            sb.loc[slot] = loc;
        }
        __syncwarp();
        {
            const uint32_t qn = base + bstride + (lane & (parts - 1));
            if (qn < total) rec = sorted[seg_index(qn, seg_begin, seg_pref, nseg)];
        }
        const int np = min((uint32_t)parts, total - base);
        if (fast)
            deposit_all<WIDE, true>(acc, sb, np, NGS, lane);
        else
            deposit_all<WIDE, false>(acc, sb, np, NGS, lane);
        __syncwarp();
    }
}

// Persistent: each CTA paints tiles blockIdx.x, blockIdx.x + gridDim.x, ...
// The next tile's segment offsets are loaded during the write-out, the
// accumulators are cleared as they are written out, and each warp loads its
// next batch of records before depositing the current one.
// NGR = pp.ngrids (1 or 2), a template parameter so that the staging and
// deposit loops are specialised for one grid or the interlaced pair.
template <int NGR>
__global__ void __launch_bounds__(kPaintThreads, 2)
paint_coop_kernel(PaintParams pp, const uint32_t *__restrict__ off, const uint4 *__restrict__ sorted,
                  PaintOut po, unsigned ntiles, int gsplit) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    uint32_t *acc = reinterpret_cast<uint32_t *>(smem_raw);                 // [2][kGS]
    StageBuf *stage = reinterpret_cast<StageBuf *>(smem_raw + kAccBytes);  // [warps]
    // the per-block counts and their window sums (before pass B) use the stage area
    uint32_t *blk = reinterpret_cast<uint32_t *>(stage) + kBlkN;  // [kBlkN]
    static_assert(2 * kBlkN * sizeof(uint32_t) <= sizeof(StageBuf) * (kPaintThreads / 32), "block counts");
    __shared__ uint32_t seg_begin[kMaxSeg];
    __shared__ uint32_t seg_pref[kMaxSeg + 1];
    __shared__ uint32_t scan_ws[33];
    __shared__ int fixbits_s;
    // packed local indices of the 4 stencil cells along i and j for a first
    // cell at l = -4 .. 35 relative to the tile start (kOut outside the tile);
    // they depend only on the tile extent, so they are rebuilt only when it changes
    __shared__ uint32_t loctab[2][40];
    // and as row masks: bit a (one bit per nibble for i, for the product with
    // the j mask) set when stencil row a lies inside the tile
    __shared__ uint32_t masktab[2][40];
    int tab_te0 = -1, tab_te1 = -1;
    // rebuild the tables for tile extents te0 x te1 (if they changed)
    auto build_tabs = [&](int te0, int te1) {
        if (te0 == tab_te0 && te1 == tab_te1) return;
        __syncthreads();
        if (threadIdx.x < 80) {
            const int a = threadIdx.x / 40, l = threadIdx.x % 40 - 4, te = a == 0 ? te0 : te1;
            uint32_t v = 0, m = 0;
#pragma unroll
            for (int s4 = 0; s4 < 4; ++s4) {
                const bool in = (unsigned)(l + s4) < (unsigned)te;
                v |= (in ? (uint32_t)(l + s4) : kOut) << (8 * s4);
                m |= (in ? 1u : 0u) << (a == 0 ? 4 * s4 : s4);
            }
            loctab[a][l + 4] = v;
            masktab[a][l + 4] = m;
        }
        __syncthreads();
        tab_te0 = te0;
        tab_te1 = te1;
    };

    const int Ng = pp.Ng, ngr = NGR;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarp = kPaintThreads / 32;  // launched with kPaintThreads
    // gsplit (NGR = 1 with pp.ngrids = 2): even CTAs paint grid 0 and odd
    // CTAs grid 1 of the same tiles, from one sort keyed for both grids
    const int mg = (NGR == 1 && gsplit) ? (int)(blockIdx.x & 1) : 0;  // the grid of a one-grid CTA
    const unsigned cta = (NGR == 1 && gsplit) ? blockIdx.x >> 1 : blockIdx.x;
    const unsigned ncta = (NGR == 1 && gsplit) ? gridDim.x >> 1 : gridDim.x;
    unsigned tile = cta;
    if (tile >= ntiles) return;
    for (int e = tid; e < (int)(kAccBytes / 16); e += kPaintThreads)
        reinterpret_cast<uint4 *>(smem_raw)[e] = make_uint4(0, 0, 0, 0);
    TileSegs ts;
    {
        uint32_t b, cnt;
        const int ncomb = tile_segment(pp, off, tile, tid, b, cnt);
        tile_publish(ncomb, b, cnt, seg_begin, seg_pref, scan_ws, ts);  // also orders the clearing above
    }
    const int fb = pp.fb;
    for (;;) {
        tile_geometry(pp, tile, ts);
        const uint32_t total = ts.total;
        const int nseg = ts.nseg;
        bool cyc[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) cyc[a] = ts.te[a] == Ng;
        build_tabs(ts.te[0], ts.te[1]);

        // fixed-point scale: the tile's particle total bounds every cell's
        // contributor count; only when that bound leaves fewer than
        // kBlockCountBelow bits are the particles counted per 4^3 block of grid-0 base cells (over the tile
        // plus a 4-cell margin, or the whole periodic axis when one tile spans it)
        int fixbits = fix_bits_for(total);
        if (fixbits < kBlockCountBelow) {
            int nb[3];
#pragma unroll
            for (int a = 0; a < 3; ++a) nb[a] = cyc[a] ? (Ng + kBlk - 1) / kBlk : blk_dim(a);
            for (int e = tid; e < kBlkN; e += kPaintThreads) blk[e] = 0u;
            __syncthreads();
            for (uint32_t q = tid; q < total; q += kPaintThreads) {
                const uint4 r = sorted[seg_index(q, seg_begin, seg_pref, nseg)];
                const uint32_t rw[3] = {r.x, r.y, r.z};
                int bidx = 0;
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    const int b = (int)(rw[a] >> fb);
                    int bb;
                    if (cyc[a]) {
                        bb = b / kBlk;
                    } else {
                        int l = b - ts.t0[a];
                        if (l > Ng / 2) l -= Ng;
                        if (l < -Ng / 2) l += Ng;
                        bb = (l + 4) / kBlk;  // margin of 4 cells below the tile
                        bb = bb < 0 ? 0 : (bb >= nb[a] ? nb[a] - 1 : bb);
                    }
                    bidx = bidx * blk_dim(a) + bb;
                }
                atomicAdd(&blk[bidx], 1u);
            }
            __syncthreads();
            // A cell's contributors have grid-0 base cells from 3 below to 3
            // above it per axis, within 3 consecutive blocks (cyclically on a
            // periodic axis): the largest 3x3x3 block sum bounds every cell's
            // contributor count.  Separable window sums along k, j, i; tmp
            // reuses the stage area.
            uint32_t *tmp = reinterpret_cast<uint32_t *>(stage);
            const int D1 = blk_dim(1), D2 = blk_dim(2);
            for (int e = tid; e < kBlkN; e += kPaintThreads) {
                const int k = e % D2, j = (e / D2) % D1, i = e / (D2 * D1);
                uint32_t v = 0;
                const bool in = i < nb[0] && j < nb[1] && k < nb[2] && (cyc[2] || k + 2 < nb[2]);
                if (in)
                    for (int c = 0; c < 3; ++c) v += blk[(i * D1 + j) * D2 + (cyc[2] ? (k + c) % nb[2] : k + c)];
                tmp[e] = v;
            }
            __syncthreads();
            for (int e = tid; e < kBlkN; e += kPaintThreads) {
                const int k = e % D2, j = (e / D2) % D1, i = e / (D2 * D1);
                uint32_t v = 0;
                const bool in = i < nb[0] && j < nb[1] && k < nb[2] && (cyc[1] || j + 2 < nb[1]);
                if (in)
                    for (int c = 0; c < 3; ++c) v += tmp[(i * D1 + (cyc[1] ? (j + c) % nb[1] : j + c)) * D2 + k];
                blk[e] = v;
            }
            __syncthreads();
            uint32_t mx = 0;
            for (int e = tid; e < kBlkN; e += kPaintThreads) {
                const int k = e % D2, j = (e / D2) % D1, i = e / (D2 * D1);
                const bool in = i < nb[0] && j < nb[1] && k < nb[2] && (cyc[0] || i + 2 < nb[0]);
                if (in) {
                    uint32_t v = 0;
                    for (int c = 0; c < 3; ++c) v += blk[((cyc[0] ? (i + c) % nb[0] : i + c) * D1 + j) * D2 + k];
                    mx = max(mx, v);
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
            if (lane == 0) scan_ws[warp] = mx;
            __syncthreads();
            if (tid == 0) {
                uint32_t m = 0;
                for (int w = 0; w < nwarp; ++w) m = max(m, scan_ws[w]);
                fixbits_s = fix_bits_for(m);
            }
            __syncthreads();
            fixbits = fixbits_s;
        }
        // a dense tile paints one grid per pass into 64-bit sums (one half of
        // a 32-row tile at a time: 16 rows of 64-bit sums fill the shared
        // memory); otherwise one pass paints every grid into 32-bit sums
        const bool wide = fixbits < kWideBelow;
        const int nhalf = (wide && ts.te[0] > kWideRows) ? 2 : 1;
        const int npass = wide ? ngr * nhalf : 1;
        const float fscale = ldexpf(1.0f, wide ? kWideBits : fixbits);
        if (wide) {
            // the 32-bit tiles leave sums in the row padding: clear all of it
            __syncthreads();
            for (int e = tid; e < (int)(kAccBytes / 16); e += kPaintThreads)
                reinterpret_cast<uint4 *>(smem_raw)[e] = make_uint4(0, 0, 0, 0);
            __syncthreads();
        }
        const bool fast = !(cyc[0] || cyc[1] || cyc[2]);
        const unsigned next = tile + ncta;
        uint32_t nb_begin = 0, nb_cnt = 0;
        int nb_comb = 0;
        for (int pass = 0; pass < npass; ++pass) {
            const int pg = NGR == 1 ? mg : pass / nhalf;  // the grid of a wide pass
            TileSegs tv = ts;             // and its rows
            if (nhalf == 2) {
                const int ph = pass % nhalf;
                tv.t0[0] = ts.t0[0] + kWideRows * ph;
                tv.te[0] = ph ? ts.te[0] - kWideRows : kWideRows;
                build_tabs(tv.te[0], tv.te[1]);
            }
            if (wide)
                paint_records<1, true>(acc, stage[warp], sorted, seg_begin, seg_pref, tv, pp, cyc, fast, fscale, pg,
                                       loctab, masktab, lane, warp);
            else
                paint_records<NGR, false>(acc, stage[warp], sorted, seg_begin, seg_pref, ts, pp, cyc, fast, fscale,
                                                   mg, loctab, masktab, lane, warp);
            __syncthreads();

            // the next tile's segments, loaded now and published after the write-out
            if (pass == npass - 1 && next < ntiles) nb_comb = tile_segment(pp, off, next, tid, nb_begin, nb_cnt);

            // write the owned cells (and the row padding of the last k tile),
            // clearing them for the next tile: warp w writes the i rows w, w + 16,
            // ..., stepping along j with pointer increments; lanes along k
            {
                const bool last_k = (ts.t0[2] + ts.te[2] == Ng);
                const int rowlen = ts.te[2] + (last_k ? pp.Ng_pad - Ng : 0);
                const int te1 = ts.te[1], te2 = ts.te[2];
                const long rstride = (long)pp.Ng_pad;  // global floats between consecutive j
                const long istride = rstride * Ng;     // and between consecutive i
                const double s0 = po.ds ? po.ds->scale[0] : po.scale[0], s1 = po.ds ? po.ds->scale[1] : po.scale[1];
                const long obase = ((long)ts.t0[0] * Ng + ts.t0[1]) * rstride + ts.t0[2];
                if (wide) {
                    // grid pg's rows of this pass from the 64-bit sums, then clear them all
                    const double scd = ldexp(pg == 0 ? s0 : s1, -kWideBits);
                    const float scf = (float)scd;
                    const int accu = po.accumulate[pg];
                    const unsigned long long *acc64 = reinterpret_cast<const unsigned long long *>(acc);
                    const long vbase = ((long)tv.t0[0] * Ng + tv.t0[1]) * rstride + tv.t0[2];
                    for (int li = warp; li < tv.te[0]; li += nwarp) {
                        float *o = reinterpret_cast<float *>(po.out[pg]) + vbase + li * istride;
                        const unsigned long long *a = acc64 + kPadK + li * kSI;
                        for (int lj = 0; lj < te1; ++lj, o += rstride, a += kSJ) {
                            float v = 0.f * scf;
                            if (lane < te2) v = (float)((double)a[lane] * scd);
                            if (lane < rowlen) {
                                if (!accu) o[lane] = v;
                                else if (lane < te2) o[lane] += v;
                            }
                            if (lane + 32 < rowlen && !accu) o[lane + 32] = 0.f * scf;
                        }
                    }
                    __syncthreads();
                    for (int e = tid; e < (int)(kAccBytes / 16); e += kPaintThreads)
                        reinterpret_cast<uint4 *>(smem_raw)[e] = make_uint4(0, 0, 0, 0);
                    __syncthreads();
                    continue;
                }
                // grid 0 here is the CTA's grid mg when it paints one grid
                const float sc0 = (float)ldexp(mg ? s1 : s0, -fixbits);
                const float sc1 = ngr > 1 ? (float)ldexp(s1, -fixbits) : 0.f;
                const int accu0 = po.accumulate[mg];
                for (int li = warp; li < ts.te[0]; li += nwarp) {
                    float *o0 = reinterpret_cast<float *>(po.out[mg]) + obase + li * istride;
                    float *o1 = ngr > 1 ? reinterpret_cast<float *>(po.out[1]) + obase + li * istride : nullptr;
                    uint32_t *a0 = acc + kPadK + li * kSI;
                    uint32_t *a1 = a0 + kGS;
                    for (int lj = 0; lj < te1; ++lj, o0 += rstride, o1 += rstride, a0 += kSJ, a1 += kSJ) {
                        // padding cells take 0 x scale, as the reference scales the
                        // whole padded grid (src/fft.c:127-129): NaN for an empty catalog
                        float v0 = 0.f * sc0, v1 = 0.f * sc1;
                        if (lane < te2) {
                            const uint32_t c0 = a0[lane];
                            a0[lane] = 0u;
                            v0 = __uint2float_rn(c0) * sc0;
                            if (ngr > 1) {
                                const uint32_t c1 = a1[lane];
                                a1[lane] = 0u;
                                v1 = __uint2float_rn(c1) * sc1;
                            }
                        }
                        if (lane < rowlen) {
                            if (!accu0) o0[lane] = v0;
                            else if (lane < te2) o0[lane] += v0;
                            if (ngr > 1) {
                                if (!po.accumulate[1]) o1[lane] = v1;
                                else if (lane < te2) o1[lane] += v1;
                            }
                        }
                        if (lane + 32 < rowlen) {  // row padding beyond a full 32-cell tile
                            if (!accu0) o0[lane + 32] = 0.f * sc0;
                            if (ngr > 1 && !po.accumulate[1]) o1[lane + 32] = 0.f * sc1;
                        }
                    }
                }
            }
        }
        if (next >= ntiles) break;
        // the clearing above completes before the next deposit: tile_publish
        // synchronises the CTA
        tile_publish(nb_comb, nb_begin, nb_cnt, seg_begin, seg_pref, scan_ws, ts);
        tile = next;
    }
}

// FP64 grids: one thread per particle, FP64 shared atomics
__global__ void __launch_bounds__(kPaintThreads)
paint_tile_f64_kernel(PaintParams pp, const uint32_t *__restrict__ off,
                      const Rec<double>::type *__restrict__ sorted, PaintOut po) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double *acc = reinterpret_cast<double *>(smem_raw);  // [ngrids][kT3], dense [16][16][32]
    __shared__ uint32_t seg_begin[kMaxSeg];
    __shared__ uint32_t seg_pref[kMaxSeg + 1];
    __shared__ uint32_t scan_ws[33];
    const int Ng = pp.Ng, ngr = pp.ngrids;
    for (int e = threadIdx.x; e < ngr * kT3; e += blockDim.x) acc[e] = 0.0;
    TileSegs ts;
    tile_segments(pp, off, seg_begin, seg_pref, scan_ws, ts);
    for (uint32_t q = threadIdx.x; q < ts.total; q += blockDim.x) {
        const auto r = sorted[seg_index(q, seg_begin, seg_pref, ts.nseg)];
        const double pos[3] = {r.x, r.y, r.z};
        for (int g = 0; g < ngr; ++g) {
            int loc[3][4];
            double w[3][4];
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                int b;
                double d;
                coord(pos[a], pp.ax[a], g, Ng, b, d);
                pcs_weights(d, w[a]);
#pragma unroll
                for (int s = 0; s < 4; ++s) loc[a][s] = local_cell(b, s, Ng, ts.t0[a], ts.te[a]);
            }
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                if (loc[0][i] < 0) continue;
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    if (loc[1][j] < 0) continue;
                    const double wij = __dmul_rn(w[0][i], w[1][j]);
                    double *row = acc + g * kT3 + (loc[0][i] * 16 + loc[1][j]) * 32;
#pragma unroll
                    for (int k = 0; k < 4; ++k)
                        if (loc[2][k] >= 0) atomicAdd(row + loc[2][k], __dmul_rn(wij, w[2][k]));
                }
            }
        }
    }
    __syncthreads();
    const bool last_k = (ts.t0[2] + ts.te[2] == Ng);
    const int pad = last_k ? pp.Ng_pad - Ng : 0;
    const int rowlen = ts.te[2] + pad;
    const int ncell = ts.te[0] * ts.te[1] * rowlen;
    for (int g = 0; g < ngr; ++g) {
        double *out = reinterpret_cast<double *>(po.out[g]);
        const double sc = po.scale[g];
        const int accu = po.accumulate[g];
        for (int e = threadIdx.x; e < ncell; e += blockDim.x) {
            const int lk = e % rowlen, lj = (e / rowlen) % ts.te[1], li = e / (rowlen * ts.te[1]);
            const long gi = ((long)(ts.t0[0] + li) * Ng + (ts.t0[1] + lj)) * pp.Ng_pad + ts.t0[2] + lk;
            // padding cells: 0 x scale, like the reference's scaling of the whole grid
            const double v = __dmul_rn(lk < ts.te[2] ? acc[g * kT3 + (li * 16 + lj) * 32 + lk] : 0.0, sc);
            if (accu) {
                if (lk < ts.te[2]) out[gi] = __dadd_rn(out[gi], v);
            } else {
                out[gi] = v;
            }
        }
    }
}

// ---- host side -----------------------------------------------------------------------------

static int tiling_build(PaintTiling *t, int Ng, const int ext[3]) {
    std::vector<int> tab;
    long nk = 27;
    for (int a = 0; a < 3; ++a) {
        int nt = (int)ceil_div(Ng, ext[a]);
        // with more than one tile per axis every extent must be >= 5 so that a
        // stencil reaches at most the adjacent tile and the classes are exclusive
        while (nt > 1 && Ng / nt < 5) --nt;
        t->tab_off[a] = (int)tab.size();
        const size_t base = tab.size();
        tab.resize(base + Ng + nt + 1);
        int tmax = 0;
        for (int q = 0; q <= nt; ++q) tab[base + Ng + q] = (int)((long)q * Ng / nt);
        for (int q = 0; q < nt; ++q) {
            const int s0 = tab[base + Ng + q], s1 = tab[base + Ng + q + 1];
            tmax = s1 - s0 > tmax ? s1 - s0 : tmax;
            for (int c = s0; c < s1; ++c) tab[base + c] = q;
        }
        if (tmax > ext[a]) return set_error(ERR_STATE, "paint tile extent %d > %d", tmax, ext[a]);
        t->nt[a] = nt;
        t->tmax[a] = tmax;
        nk *= nt;
    }
    t->Ng = Ng;
    t->nkeys = nk;
    if (t->nkeys >= (1L << 32)) return set_error(ERR_UNSUPPORTED, "too many paint tiles");
    FG_CUDA(cudaMalloc(&t->d_tables, sizeof(int) * tab.size()));
    FG_CUDA(cudaMemcpy(t->d_tables, tab.data(), sizeof(int) * tab.size(), cudaMemcpyHostToDevice));
    return OK;
}

int paint_tiling_create(PaintTiling *t, int Ng) {
    FG_TRY(tiling_build(t, Ng, kTileExt));
    if (Ng >= 64) {
        t->one = new PaintTiling();
        FG_TRY(tiling_build(t->one, Ng, kTileExt1));
    }
    return OK;
}

void paint_tiling_destroy(PaintTiling *t) {
    if (t->one) {
        paint_tiling_destroy(t->one);
        delete t->one;
        t->one = nullptr;
    }
    cudaFree(t->d_tables);
    t->d_tables = nullptr;
}

void paint_scratch_free(PaintScratch *s) {
    cudaFree(s->sorted);
    cudaFree(s->hist);
    cudaFree(s->cursor);
    cudaFree(s->scan_tmp);
    *s = PaintScratch();
}

static int ensure_scratch(PaintScratch *s, long Np, long nkeys) {
    if (Np > s->cap_particles) {
        cudaFree(s->sorted);
        s->sorted = nullptr;
        const long cap = Np + Np / 8 + 1024;
        FG_CUDA(cudaMalloc(&s->sorted, 32 * (size_t)cap));  // fits float4 and 3 doubles
        s->cap_particles = cap;
    }
    if (nkeys + 1 > s->cap_keys) {
        cudaFree(s->hist);
        cudaFree(s->cursor);
        cudaFree(s->scan_tmp);
        s->hist = s->cursor = s->scan_tmp = nullptr;
        FG_CUDA(cudaMalloc(&s->hist, sizeof(uint32_t) * (nkeys + 1)));
        FG_CUDA(cudaMalloc(&s->cursor, sizeof(uint32_t) * (nkeys + 1)));
        FG_CUDA(cudaMalloc(&s->scan_tmp, sizeof(uint32_t) * (ceil_div(nkeys + 1, kScanBlock) + 1)));
        s->cap_keys = nkeys + 1;
    }
    s->bytes = (size_t)32 * s->cap_particles + 2 * sizeof(uint32_t) * (size_t)s->cap_keys;
    return OK;
}

int paint_reserve(const PaintTiling *t, PaintScratch *s, long Np) {
    return ensure_scratch(s, Np > 0 ? Np : 1, t->nkeys);
}

static void split(double v, float &hi, float &lo) {
    hi = (float)v;
    lo = (float)(v - (double)hi);
}

int paint(const PaintTiling *t, PaintScratch *s, int grid_prec, const void *x, const void *y, const void *z,
          int pos_prec, long Np, double Hinv, const PaintGridSpec *grids, int ngrids, cudaStream_t st,
          cudaEvent_t *ev, const PaintRsd *rsd, const DevScalars *ds) {
    if (ngrids < 1 || ngrids > kMaxPaintGrids) return set_error(ERR_ARG, "paint: 1 or 2 grids");
    if (ds && (grid_prec != 4 || pos_prec != 4)) return set_error(ERR_ARG, "paint: device scalars need FP32");
    if (rsd && rsd->v[0] && pos_prec != 4) return set_error(ERR_ARG, "paint: displacement needs FP32 positions");
    if (pos_prec != grid_prec) return set_error(ERR_ARG, "paint: position precision must match grid precision");
    const int cta_per_sm = t->cta_per_sm;
    const bool big = grid_prec == 4 && t->one;  // FP32: the 32 x 16 x 32 tiles
    if (big) t = t->one;
    if (Np < 0 || Np >= (1L << 32)) return set_error(ERR_ARG, "paint: Np out of range");
    for (int g = 1; g < ngrids; ++g)
        for (int a = 0; a < 3; ++a)
            if (fabs(grids[g].offset[a] - grids[0].offset[a]) > 1.0)
                return set_error(ERR_ARG, "paint: grid offsets must lie within one cell");
    const int Ng = t->Ng;
    PaintParams pp;
    memset(&pp, 0, sizeof(pp));
    pp.Ng = Ng;
    pp.Ng_pad = 2 * (Ng / 2 + 1);
    pp.ngrids = ngrids;
    if (rsd && rsd->v[0]) {
        for (int a = 0; a < 3; ++a) {
            pp.v[a] = rsd->v[a];
            pp.los[a] = (float)rsd->los[a];
        }
        pp.aHinv = (float)rsd->aHinv;
    }
    int bits_b = 1;
    while ((1 << bits_b) < Ng) ++bits_b;
    pp.fb = 32 - bits_b < 24 ? 32 - bits_b : 24;  // 2^-24 cell: below FP32 resolution
    if (grid_prec == 4 && pp.fb < 16) return set_error(ERR_UNSUPPORTED, "FP32 paint: Ng=%d too large", Ng);
    for (int a = 0; a < 3; ++a) {
        pp.nt[a] = t->nt[a];
        pp.tile_of[a] = t->d_tables + t->tab_off[a];
        {
            const int ext = Ng / t->nt[a];
            pp.tshift[a] = -1;
            if (ext * t->nt[a] == Ng && (ext & (ext - 1)) == 0)
                for (int b = 0; (1 << b) <= ext; ++b)
                    if ((1 << b) == ext) pp.tshift[a] = b;
        }
        pp.start[a] = t->d_tables + t->tab_off[a] + Ng;
        split(Hinv, pp.ax[a].h_hi, pp.ax[a].h_lo);
        pp.ax[a].h = Hinv;
        for (int g = 0; g < ngrids; ++g) {
            split(grids[g].offset[a], pp.ax[a].o_hi[g], pp.ax[a].o_lo[g]);
            pp.ax[a].o[g] = grids[g].offset[a];
            pp.ax[a].dq[g] = (int)llrint((grids[0].offset[a] - grids[g].offset[a]) * (double)(1u << pp.fb));
        }
    }
    PaintOut po;
    memset(&po, 0, sizeof(po));
    for (int g = 0; g < ngrids; ++g) {
        po.out[g] = grids[g].out;
        po.scale[g] = grids[g].scale;
        po.accumulate[g] = grids[g].accumulate;
    }
    po.ds = ds;
    FG_TRY(ensure_scratch(s, Np > 0 ? Np : 1, t->nkeys));
    FG_CUDA(cudaMemsetAsync(s->hist, 0, sizeof(uint32_t) * (t->nkeys + 1), st));
    const int nsm = num_sms();
    const unsigned gp = (unsigned)(Np > 0 ? (ceil_div(Np, 256) < 32L * nsm ? ceil_div(Np, 256) : 32L * nsm) : 1);
    if (Np > 0) {
        if (pos_prec == 4)
            paint_key_kernel<float><<<gp, 256, 0, st>>>((const float *)x, (const float *)y, (const float *)z, Np,
                                                       pp, s->hist, ds);
        else
            paint_key_kernel<double><<<gp, 256, 0, st>>>((const double *)x, (const double *)y, (const double *)z,
                                                        Np, pp, s->hist, nullptr);
        FG_LAUNCHED(1);
    }
    if (ev) FG_CUDA(cudaEventRecord(ev[0], st));
    FG_TRY(exclusive_scan(s->hist, t->nkeys + 1, s->scan_tmp, st));
    FG_CUDA(cudaMemcpyAsync(s->cursor, s->hist, sizeof(uint32_t) * (t->nkeys + 1), cudaMemcpyDeviceToDevice, st));
    if (ev) FG_CUDA(cudaEventRecord(ev[1], st));
    if (Np > 0) {
        if (pos_prec == 4)
            paint_scatter_kernel<float><<<gp, 256, 0, st>>>((const float *)x, (const float *)y, (const float *)z,
                                                           Np, pp, s->cursor, (uint4 *)s->sorted, ds);
        else
            paint_scatter_kernel<double><<<gp, 256, 0, st>>>((const double *)x, (const double *)y,
                                                            (const double *)z, Np, pp, s->cursor,
                                                            (Rec<double>::type *)s->sorted, nullptr);
        FG_LAUNCHED(1);
    }
    if (ev) FG_CUDA(cudaEventRecord(ev[2], st));
    const unsigned ntiles = (unsigned)((long)t->nt[0] * t->nt[1] * t->nt[2]);
    if (grid_prec == 4) {
        // one grid per CTA where the tiles are 32 x 16 x 32: with two grids,
        // even CTAs paint grid 0 and odd CTAs grid 1 (the sort's keys cover
        // both grids' stencils); else both grids of 16-row tiles per CTA
        constexpr int T = kPaintThreads;
        const size_t smem = kAccBytes + sizeof(StageBuf) * (T / 32);
        FG_CUDA(cudaFuncSetAttribute(paint_coop_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        FG_CUDA(cudaFuncSetAttribute(paint_coop_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        const int split = big && ngrids == 2;
        unsigned nb = (unsigned)((cta_per_sm == 1 ? 1 : 2) * num_sms());
        if (split) {
            nb = nb < 2 * ntiles ? nb : 2 * ntiles;
            nb &= ~1u;
        } else {
            nb = nb < ntiles ? nb : ntiles;
        }
        if (ngrids == 1 || split)
            paint_coop_kernel<1><<<nb, T, smem, st>>>(pp, s->hist, (const uint4 *)s->sorted, po, ntiles, split);
        else
            paint_coop_kernel<2><<<nb, T, smem, st>>>(pp, s->hist, (const uint4 *)s->sorted, po, ntiles, 0);
    } else {
        const size_t smem = (size_t)ngrids * kT3 * sizeof(double);
        FG_CUDA(cudaFuncSetAttribute(paint_tile_f64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem));
        paint_tile_f64_kernel<<<ntiles, kPaintThreads, smem, st>>>(pp, s->hist,
                                                                    (const Rec<double>::type *)s->sorted, po);
    }
    FG_LAUNCHED(1);
    if (ev) FG_CUDA(cudaEventRecord(ev[3], st));
    return OK;
}

}  // namespace fg
