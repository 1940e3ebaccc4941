// PCS (piecewise cubic spline) mass assignment for sm_103a.
//
// Restates the arithmetic of the reference's fft_p2g (src/fft.c:57-131):
// u = x * Ng/L - offset, base cell floor(u), fraction d = u - floor(u), the four
// cubic B-spline weights of src/fft.c:83-88, cells wrapped mod Ng.  The GPU
// organisation is new:
//
//  1. key     : every particle gets the key (tile, class) of its base cell.  The
//               grid is cut into tiles of at most 16 x 16 x 32 cells (i, j, k);
//               per axis the class says whether the particle's stencil (over
//               all painted grids) reaches into the lower (1) or upper (2)
//               neighbour tile, or neither (0).  The rank of the particle
//               within its key comes from the histogram atomic.
//  2. scan    : exclusive prefix sum of the key histogram.
//  3. scatter : particles are written in key order.
//  4. paint   : one CTA per tile owns its cells.  It pulls the particles of its
//               own tile and only the boundary classes of its 26 neighbours,
//               accumulates their weights in shared memory and writes every
//               owned cell exactly once (no global atomics, no zeroing pass).
//
// FP32 grids (paint_coop_kernel): each lane prepares one particle (cell
// indices and the 3 x 4 weights of both grids) in shared memory, then the warp
// deposits the particles one at a time with lane = (grid, i row, j row), each
// lane adding its 4 k cells.  The shared layout puts those 32 rows in 32
// distinct banks.  Sums are 32-bit fixed point with a per-tile scale 2^-s: a
// first pass counts particles per 4^3-cell block, and s is the largest value
// for which no cell can exceed 2^32 (a particle adds at most (2/3)^3 of its
// weight to a cell).  Integer sums are order independent, so the painted grid
// is bit-reproducible run to run.
// FP64 grids (paint_tile_f64_kernel) reproduce the reference's FP64 weight
// arithmetic op for op and accumulate in FP64, one thread per particle.
#include "internal.h"
#include "common.cuh"

#include <math.h>
#include <string.h>
#include <vector>

namespace fg {

constexpr int kTileExt[3] = {16, 16, 32};    // i, j, k
constexpr int kMaxPaintGrids = 2;
constexpr double kMaxCellWeight = 8.0 / 27.0;  // largest PCS weight product
constexpr int kMinFixBits = 8;                 // below this: FP32 accumulation
// FP32 shared layout: cell (li, lj, lk) of grid g at g*kGS + li*kSI + lj*kSJ + lk;
// kSJ = 1, kSI = 4, kGS = 16 (mod 32) gives the 32 rows (g, li+a, lj+b),
// a, b < 4, of one stencil 32 distinct banks.  Row lj = 16 and column lk = 32
// are padding that absorbs the updates of stencil cells outside the tile, so
// the deposit needs no per-cell test.
constexpr int kSJ = 33, kSI = 580, kGS = 9264;
constexpr uint32_t kOutJ = 16, kOutK = 32;
static_assert(15 * kSI + (int)kOutJ * kSJ + (int)kOutK < kGS, "tile does not fit the layout");
static_assert(kSI % 32 == 4 && kGS % 32 == 16 && kSJ % 32 == 1, "bank layout");
// largest fixed-point scale: products stay below 2^22 so the FMA trick of
// deposit4 converts them to integers exactly
constexpr int kMaxFixBits = 23;
// FP64 shared layout: dense [16][16][32]
constexpr int kT3 = 16 * 16 * 32;
// per-tile block counts: 4^3-cell blocks over the tile plus a 4-cell margin
constexpr int kBlk = 4;
__host__ __device__ constexpr int blk_dim(int a) { return a == 2 ? (32 + 8) / kBlk : (16 + 8) / kBlk; }  // 6, 6, 10
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
    int Ng, Ng_pad, ngrids;
    int fb;                  // FP32 path: fraction bits of the packed cell coordinate
    int nt[3];
    const int *tile_of[3];   // [Ng] per axis
    const int *start[3];     // [nt + 1] per axis
};

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

template <typename P>
__global__ void paint_key_kernel(const P *__restrict__ x, const P *__restrict__ y,
                                 const P *__restrict__ z, long Np, PaintParams pp,
                                 uint32_t *__restrict__ key, uint32_t *__restrict__ rank,
                                 uint32_t *__restrict__ hist) {
    const int Ng = pp.Ng;
    for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < Np;
         p += (long)gridDim.x * blockDim.x) {
        const P pos[3] = {x[p], y[p], z[p]};
        int t[3], cls[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            int b0;
            uint32_t dq0 = 0;
            if constexpr (sizeof(P) == 4) {
                cell0(pos[a], pp.ax[a], Ng, pp.fb, b0, dq0);
            } else {
                P d;
                coord(pos[a], pp.ax[a], 0, Ng, b0, d);
            }
            const int ta = pp.tile_of[a][b0];
            const int t0 = pp.start[a][ta];
            const int te = pp.start[a][ta + 1] - t0;
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
                const int dl = ((bg - b0 + Ng + 1) % Ng) - 1;  // -1, 0 or +1
                rmin = min(rmin, b0 - t0 + dl);
                rmax = max(rmax, b0 - t0 + dl);
            }
            t[a] = ta;
            cls[a] = pp.nt[a] == 1 ? 0 : (rmin - 1 < 0 ? 1 : (rmax + 2 >= te ? 2 : 0));
        }
        const uint32_t k = (uint32_t)((((long)t[0] * pp.nt[1] + t[1]) * pp.nt[2] + t[2]) * 27 + cls[0] * 9 +
                                      cls[1] * 3 + cls[2]);
        key[p] = k;
        rank[p] = atomicAdd(&hist[k], 1u);
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
                                     const uint32_t *__restrict__ key,
                                     const uint32_t *__restrict__ rank,
                                     const uint32_t *__restrict__ off,
                                     typename Rec<P>::type *__restrict__ sorted) {
    for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < Np;
         p += (long)gridDim.x * blockDim.x) {
        const uint32_t dst = off[key[p]] + rank[p];
        typename Rec<P>::type r;
        if constexpr (sizeof(P) == 4) {
            const float pos[3] = {x[p], y[p], z[p]};
            uint32_t w[3];
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                int b0;
                uint32_t dq;
                cell0(pos[a], pp.ax[a], pp.Ng, pp.fb, b0, dq);
                w[a] = ((uint32_t)b0 << pp.fb) | dq;
            }
            r = make_uint4(w[0], w[1], w[2], 0u);
        } else {
            r.x = x[p];
            r.y = y[p];
            r.z = z[p];
        }
        sorted[dst] = r;
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
};

// Tile geometry and the flattened list of particle segments a tile pulls:
// its own key range for every class and the boundary classes of the (up to
// 26, deduplicated for 1 or 2 tiles per axis) neighbours.
struct TileSegs {
    int t0[3], te[3];
    int nseg;
    uint32_t total;
};

__device__ void tile_segments(const PaintParams &pp, const uint32_t *__restrict__ off, uint32_t *seg_begin,
                              uint32_t *seg_pref, uint32_t *scan_ws, TileSegs &ts) {
    const int nt0 = pp.nt[0], nt1 = pp.nt[1], nt2 = pp.nt[2];
    const int tt[3] = {(int)(blockIdx.x / (nt1 * nt2)), (int)((blockIdx.x / nt2) % nt1), (int)(blockIdx.x % nt2)};
    (void)nt0;
    int nopt[3], otile[3][5], ocls[3][5];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        ts.t0[a] = pp.start[a][tt[a]];
        ts.te[a] = pp.start[a][tt[a] + 1] - ts.t0[a];
        const int nt = pp.nt[a];
        int k = 0;
        if (nt == 1) {
            otile[a][k] = tt[a];
            ocls[a][k++] = 0;
        } else {
            for (int c = 0; c < 3; ++c) {
                otile[a][k] = tt[a];
                ocls[a][k++] = c;
            }
            const int lo = (tt[a] + nt - 1) % nt, hi = (tt[a] + 1) % nt;
            if (nt == 2) {
                otile[a][k] = hi;
                ocls[a][k++] = 1;
                otile[a][k] = hi;
                ocls[a][k++] = 2;
            } else {
                otile[a][k] = lo;  // lower tile, particles reaching up
                ocls[a][k++] = 2;
                otile[a][k] = hi;  // upper tile, particles reaching down
                ocls[a][k++] = 1;
            }
        }
        nopt[a] = k;
    }
    const int ncomb = nopt[0] * nopt[1] * nopt[2];  // <= 125
    const int q = threadIdx.x;
    uint32_t b = 0, cnt = 0;
    if (q < ncomb) {
        const int i = q / (nopt[1] * nopt[2]), j = (q / nopt[2]) % nopt[1], k = q % nopt[2];
        const long key = (((long)otile[0][i] * nt1 + otile[1][j]) * nt2 + otile[2][k]) * 27 + ocls[0][i] * 9 +
                         ocls[1][j] * 3 + ocls[2][k];
        b = off[key];
        cnt = off[key + 1] - b;
    }
    uint32_t tot;
    const uint32_t pref = block_exclusive_scan(cnt, scan_ws, &scan_ws[31]);
    tot = scan_ws[31];
    if (q < ncomb) {
        seg_begin[q] = b;
        seg_pref[q] = pref;
    }
    if (q == 0) seg_pref[ncomb] = tot;
    __syncthreads();
    ts.nseg = ncomb;
    ts.total = seg_pref[ncomb];
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

struct __align__(16) StageRec {
    uint32_t loc[4];  // per axis: 4 packed local cell indices (255 = outside the tile); [3] unused
    float4 w[3];      // per axis: PCS weights (k weights pre-scaled by 2^s)
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

// deposit staged particles one at a time: lane = (grid, i row, j row), every
// lane adds its row's 4 k cells.  By the bank layout the 32 rows of one
// particle start in 32 distinct banks, so each of the 4 atomics is a single
// shared-memory wavefront (the limiting resource of this kernel).  Cells
// outside the tile land in the padding row / column.
template <bool FIXED>
__device__ __forceinline__ void deposit_all(uint32_t *acc, const StageRec *mystage, int np, int ngr, int lane) {
    const int g = lane >> 4, a = (lane >> 2) & 3, b = lane & 3;
    if (g >= ngr) return;
    const float M = 12582912.0f;  // 1.5 * 2^23: FMA onto it rounds w to an integer
    for (int p = 0; p < np; ++p) {
        const StageRec &st = mystage[p * kMaxPaintGrids + g];
        const uint4 loc = *reinterpret_cast<const uint4 *>(st.loc);
        const uint32_t li = (loc.x >> (8 * a)) & 255u;
        if (li == 255u) continue;
        const uint32_t lj = (loc.y >> (8 * b)) & 255u;
        uint32_t *row = acc + g * kGS + li * kSI + lj * kSJ;
        const float w = reinterpret_cast<const float *>(&st.w[0])[a] * reinterpret_cast<const float *>(&st.w[1])[b];
        const float4 wz = st.w[2];
        const uint32_t k0 = loc.z & 255u, k1 = (loc.z >> 8) & 255u, k2 = (loc.z >> 16) & 255u, k3 = loc.z >> 24;
        if (FIXED) {
            atomicAdd(row + k0, __float_as_uint(fmaf(w, wz.x, M)) - 0x4B400000u);
            atomicAdd(row + k1, __float_as_uint(fmaf(w, wz.y, M)) - 0x4B400000u);
            atomicAdd(row + k2, __float_as_uint(fmaf(w, wz.z, M)) - 0x4B400000u);
            atomicAdd(row + k3, __float_as_uint(fmaf(w, wz.w, M)) - 0x4B400000u);
        } else {
            float *rowf = reinterpret_cast<float *>(row);
            atomicAdd(rowf + k0, w * wz.x);
            atomicAdd(rowf + k1, w * wz.y);
            atomicAdd(rowf + k2, w * wz.z);
            atomicAdd(rowf + k3, w * wz.w);
        }
    }
}

__global__ void __launch_bounds__(kPaintThreads, 2)
paint_coop_kernel(PaintParams pp, const uint32_t *__restrict__ off, const uint4 *__restrict__ sorted,
                  PaintOut po) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    uint32_t *acc = reinterpret_cast<uint32_t *>(smem_raw);                       // [2][kGS]
    StageRec *stage = reinterpret_cast<StageRec *>(acc + kMaxPaintGrids * kGS);  // [warps][16][grids]
    uint32_t *blk = reinterpret_cast<uint32_t *>(stage + (kPaintThreads / 32) * kStageParts * kMaxPaintGrids);  // [kBlkN]
    __shared__ uint32_t seg_begin[kMaxSeg];
    __shared__ uint32_t seg_pref[kMaxSeg + 1];
    __shared__ uint32_t scan_ws[32];
    __shared__ int fixbits_s;

    const int Ng = pp.Ng, ngr = pp.ngrids;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarp = blockDim.x >> 5;
    for (int e = tid; e < ngr * kGS / 4; e += blockDim.x) reinterpret_cast<uint4 *>(acc)[e] = make_uint4(0, 0, 0, 0);
    for (int e = tid; e < kBlkN; e += blockDim.x) blk[e] = 0u;
    TileSegs ts;
    tile_segments(pp, off, seg_begin, seg_pref, scan_ws, ts);
    const uint32_t total = ts.total;
    const int nseg = ts.nseg;

    // pass A: particles per 4^3 block of grid-0 base cells.  Along an axis cut
    // into several tiles the blocks cover the tile plus a 4-cell margin; along
    // an axis held by a single tile they tile the periodic axis itself.
    int nb[3];
    bool cyc[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        cyc[a] = ts.te[a] == Ng;
        nb[a] = cyc[a] ? (Ng + kBlk - 1) / kBlk : blk_dim(a);
    }
    const int fb = pp.fb;
    for (uint32_t q = tid; q < total; q += blockDim.x) {
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
    // A cell's contributors have grid-0 base cells from 3 below to 3 above it
    // per axis, within 3 consecutive blocks (cyclically on a periodic axis):
    // the largest 3x3x3 block sum bounds every cell's contributor count.
    // Separable window sums along k, then j, then i; tmp reuses the stage area.
    {
        uint32_t *tmp = reinterpret_cast<uint32_t *>(stage);
        const int D1 = blk_dim(1), D2 = blk_dim(2);
        for (int e = tid; e < kBlkN; e += blockDim.x) {
            const int k = e % D2, j = (e / D2) % D1, i = e / (D2 * D1);
            uint32_t v = 0;
            const bool in = i < nb[0] && j < nb[1] && k < nb[2] && (cyc[2] || k + 2 < nb[2]);
            if (in)
                for (int c = 0; c < 3; ++c) v += blk[(i * D1 + j) * D2 + (cyc[2] ? (k + c) % nb[2] : k + c)];
            tmp[e] = v;
        }
        __syncthreads();
        for (int e = tid; e < kBlkN; e += blockDim.x) {
            const int k = e % D2, j = (e / D2) % D1, i = e / (D2 * D1);
            uint32_t v = 0;
            const bool in = i < nb[0] && j < nb[1] && k < nb[2] && (cyc[1] || j + 2 < nb[1]);
            if (in)
                for (int c = 0; c < 3; ++c) v += tmp[(i * D1 + (cyc[1] ? (j + c) % nb[1] : j + c)) * D2 + k];
            blk[e] = v;
        }
        __syncthreads();
        uint32_t mx = 0;
        for (int e = tid; e < kBlkN; e += blockDim.x) {
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
            int fb = kMaxFixBits;
            if (m > 0) fb = (int)floor(log2(4294967295.0 / ((double)m * kMaxCellWeight)));
            fixbits_s = fb > kMaxFixBits ? kMaxFixBits : fb;
        }
    }
    __syncthreads();
    const int fixbits = fixbits_s;
    const bool fixed = fixbits >= kMinFixBits;
    const float fscale = ldexpf(1.0f, fixed ? fixbits : 0);

    // pass B: stage 32 particles per warp, then deposit them one by one
    StageRec *mystage = stage + warp * kStageParts * kMaxPaintGrids;
    for (uint32_t base = (uint32_t)warp * kStageParts; base < total; base += (uint32_t)nwarp * kStageParts) {
        const uint32_t q = base + (lane & (kStageParts - 1));
        const int gs = lane / kStageParts;  // lanes 0..15 stage grid 0, 16..31 grid 1
        if (q < total && gs < ngr) {
            const uint4 r = sorted[seg_index(q, seg_begin, seg_pref, nseg)];
            const uint32_t rw[3] = {r.x, r.y, r.z};
            StageRec &st = mystage[(lane & (kStageParts - 1)) * kMaxPaintGrids + gs];
            const float inv = ldexpf(1.0f, -fb);
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                int bg;
                uint32_t dgq;
                cell_g((int)(rw[a] >> fb), rw[a] & ((1u << fb) - 1), pp.ax[a].dq[gs], fb, Ng, bg, dgq);
                float w[4];
                pcs_weights((float)dgq * inv, w);
                const uint32_t outv = a == 0 ? 255u : (a == 1 ? kOutJ : kOutK);
                uint32_t loc;
                if (cyc[a]) {
                    loc = pack_local(bg, Ng, ts.t0[a], ts.te[a], outv);
                } else {
                    // linear local index of the first stencil cell (periodic
                    // images folded to the nearest copy of the tile)
                    int l = bg - 1 - ts.t0[a];
                    l -= l > Ng / 2 ? Ng : 0;
                    l += l < -Ng / 2 ? Ng : 0;
                    loc = 0;
#pragma unroll
                    for (int s4 = 0; s4 < 4; ++s4)
                        loc |= ((unsigned)(l + s4) < (unsigned)ts.te[a] ? (uint32_t)(l + s4) : outv) << (8 * s4);
                }
                st.loc[a] = loc;
                const float sc = a == 2 ? fscale : 1.f;
                st.w[a] = make_float4(w[0] * sc, w[1] * sc, w[2] * sc, w[3] * sc);
            }
        }
        __syncwarp();
        const int np = min((uint32_t)kStageParts, total - base);
        if (fixed)
            deposit_all<true>(acc, mystage, np, ngr, lane);
        else
            deposit_all<false>(acc, mystage, np, ngr, lane);
        __syncwarp();
    }
    __syncthreads();

    // write the owned cells (and the row padding of the last k tile): one
    // warp per (i, j) row, lanes along k, rows advanced incrementally
    const bool last_k = (ts.t0[2] + ts.te[2] == Ng);
    const int pad = last_k ? pp.Ng_pad - Ng : 0;
    const int rowlen = ts.te[2] + pad, te1 = ts.te[1], te2 = ts.te[2];
    const int nrow = ts.te[0] * te1;
    const long rstride = (long)pp.Ng_pad;  // global floats between consecutive j
    for (int g = 0; g < ngr; ++g) {
        float *out = reinterpret_cast<float *>(po.out[g]) + ((long)ts.t0[0] * Ng + ts.t0[1]) * rstride + ts.t0[2];
        const float sc = (float)ldexp(po.scale[g], fixed ? -fixbits : 0);
        const bool accu = po.accumulate[g] != 0;
        int li = warp / te1, lj = warp - li * te1;
        const int dli = nwarp / te1, dlj = nwarp - dli * te1;
        for (int r = warp; r < nrow; r += nwarp) {
            float *orow = out + ((long)li * Ng + lj) * rstride;
            const uint32_t *arow = acc + g * kGS + li * kSI + lj * kSJ;
            for (int lk = lane; lk < rowlen; lk += 32) {
                float v = 0.f;
                if (lk < te2) {
                    const uint32_t a = arow[lk];
                    v = (fixed ? __uint2float_rn(a) : __uint_as_float(a)) * sc;
                }
                if (!accu)
                    orow[lk] = v;
                else if (lk < te2)
                    orow[lk] += v;
            }
            li += dli;
            lj += dlj;
            if (lj >= te1) {
                lj -= te1;
                ++li;
            }
        }
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
    __shared__ uint32_t scan_ws[32];
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
            double v = 0;
            if (lk < ts.te[2]) v = __dmul_rn(acc[g * kT3 + (li * 16 + lj) * 32 + lk], sc);
            if (accu) {
                if (lk < ts.te[2]) out[gi] = __dadd_rn(out[gi], v);
            } else {
                out[gi] = v;
            }
        }
    }
}

// ---- host side -----------------------------------------------------------------------------

int paint_tiling_create(PaintTiling *t, int Ng) {
    std::vector<int> tab;
    long nk = 27;
    for (int a = 0; a < 3; ++a) {
        int nt = (int)ceil_div(Ng, kTileExt[a]);
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
        if (tmax > kTileExt[a]) return set_error(ERR_STATE, "paint tile extent %d > %d", tmax, kTileExt[a]);
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

void paint_tiling_destroy(PaintTiling *t) {
    cudaFree(t->d_tables);
    t->d_tables = nullptr;
}

void paint_scratch_free(PaintScratch *s) {
    cudaFree(s->key);
    cudaFree(s->rank);
    cudaFree(s->sorted);
    cudaFree(s->hist);
    cudaFree(s->scan_tmp);
    *s = PaintScratch();
}

static int ensure_scratch(PaintScratch *s, long Np, long nkeys) {
    if (Np > s->cap_particles) {
        cudaFree(s->key);
        cudaFree(s->rank);
        cudaFree(s->sorted);
        s->key = s->rank = nullptr;
        s->sorted = nullptr;
        const long cap = Np + Np / 8 + 1024;
        FG_CUDA(cudaMalloc(&s->key, sizeof(uint32_t) * cap));
        FG_CUDA(cudaMalloc(&s->rank, sizeof(uint32_t) * cap));
        FG_CUDA(cudaMalloc(&s->sorted, 32 * (size_t)cap));  // fits float4 and 3 doubles
        s->cap_particles = cap;
    }
    if (nkeys + 1 > s->cap_keys) {
        cudaFree(s->hist);
        cudaFree(s->scan_tmp);
        s->hist = s->scan_tmp = nullptr;
        FG_CUDA(cudaMalloc(&s->hist, sizeof(uint32_t) * (nkeys + 1)));
        FG_CUDA(cudaMalloc(&s->scan_tmp, sizeof(uint32_t) * (ceil_div(nkeys + 1, kScanBlock) + 1)));
        s->cap_keys = nkeys + 1;
    }
    s->bytes = (sizeof(uint32_t) * 2 + 32) * (size_t)s->cap_particles + sizeof(uint32_t) * (size_t)s->cap_keys;
    return OK;
}

static void split(double v, float &hi, float &lo) {
    hi = (float)v;
    lo = (float)(v - (double)hi);
}

int paint(const PaintTiling *t, PaintScratch *s, int grid_prec, const void *x, const void *y, const void *z,
          int pos_prec, long Np, double Hinv, const PaintGridSpec *grids, int ngrids, cudaStream_t st,
          cudaEvent_t *ev) {
    if (ngrids < 1 || ngrids > kMaxPaintGrids) return set_error(ERR_ARG, "paint: 1 or 2 grids");
    if (pos_prec != grid_prec) return set_error(ERR_ARG, "paint: position precision must match grid precision");
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
    int bits_b = 1;
    while ((1 << bits_b) < Ng) ++bits_b;
    pp.fb = 32 - bits_b < 24 ? 32 - bits_b : 24;  // 2^-24 cell: below FP32 resolution
    if (grid_prec == 4 && pp.fb < 16) return set_error(ERR_UNSUPPORTED, "FP32 paint: Ng=%d too large", Ng);
    for (int a = 0; a < 3; ++a) {
        pp.nt[a] = t->nt[a];
        pp.tile_of[a] = t->d_tables + t->tab_off[a];
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
    FG_TRY(ensure_scratch(s, Np > 0 ? Np : 1, t->nkeys));
    FG_CUDA(cudaMemsetAsync(s->hist, 0, sizeof(uint32_t) * (t->nkeys + 1), st));
    const int nsm = num_sms();
    const unsigned gp = (unsigned)(Np > 0 ? (ceil_div(Np, 256) < 32L * nsm ? ceil_div(Np, 256) : 32L * nsm) : 1);
    if (Np > 0) {
        if (pos_prec == 4)
            paint_key_kernel<float><<<gp, 256, 0, st>>>((const float *)x, (const float *)y, (const float *)z, Np,
                                                       pp, s->key, s->rank, s->hist);
        else
            paint_key_kernel<double><<<gp, 256, 0, st>>>((const double *)x, (const double *)y, (const double *)z,
                                                        Np, pp, s->key, s->rank, s->hist);
        FG_LAUNCHED(1);
    }
    if (ev) FG_CUDA(cudaEventRecord(ev[0], st));
    FG_TRY(exclusive_scan(s->hist, t->nkeys + 1, s->scan_tmp, st));
    if (ev) FG_CUDA(cudaEventRecord(ev[1], st));
    if (Np > 0) {
        if (pos_prec == 4)
            paint_scatter_kernel<float><<<gp, 256, 0, st>>>((const float *)x, (const float *)y, (const float *)z,
                                                           Np, pp, s->key, s->rank, s->hist, (uint4 *)s->sorted);
        else
            paint_scatter_kernel<double><<<gp, 256, 0, st>>>((const double *)x, (const double *)y,
                                                            (const double *)z, Np, pp, s->key, s->rank, s->hist,
                                                            (Rec<double>::type *)s->sorted);
        FG_LAUNCHED(1);
    }
    if (ev) FG_CUDA(cudaEventRecord(ev[2], st));
    const unsigned ntiles = (unsigned)((long)t->nt[0] * t->nt[1] * t->nt[2]);
    if (grid_prec == 4) {
        const size_t smem = sizeof(uint32_t) * kMaxPaintGrids * kGS +
                            sizeof(StageRec) * (kPaintThreads / 32) * kStageParts * kMaxPaintGrids +
                            sizeof(uint32_t) * kBlkN;
        FG_CUDA(cudaFuncSetAttribute(paint_coop_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        paint_coop_kernel<<<ntiles, kPaintThreads, smem, st>>>(pp, s->hist, (const uint4 *)s->sorted, po);
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
