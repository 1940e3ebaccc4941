// PCS (piecewise cubic spline) mass assignment for sm_103a.
//
// Restates the arithmetic of the reference's fft_p2g (src/fft.c:57-131):
// u = x * Ng/L - offset, base cell floor(u), fraction d = u - floor(u), the four
// cubic B-spline weights of src/fft.c:83-88, cells wrapped mod Ng.  The GPU
// organisation is new:
//
//  1. key     : every particle gets the key (tile, class) of its base cell.  The
//               grid is cut into <= 16^3-cell tiles; per axis the class says
//               whether the particle's stencil (over all painted grids) reaches
//               into the lower (1) or upper (2) neighbour tile, or neither (0).
//               The rank of the particle within its key comes from the
//               histogram atomic.
//  2. scan    : exclusive prefix sum of the key histogram.
//  3. scatter : particles are written in key order.
//  4. paint   : one CTA per tile owns its cells.  It pulls the particles of its
//               own tile and only the boundary classes of its 26 neighbours,
//               accumulates their weights in shared memory and writes every
//               owned cell exactly once (no global atomics, no zeroing pass).
//
// FP32 grids accumulate in 32-bit fixed point with a per-tile scale 2^-s,
// s chosen from the tile's particle count so that no cell sum can overflow
// (a particle adds at most (2/3)^3 of its weight to one cell).  Integer sums
// are order independent, so the painted grid is bit-reproducible run to run;
// 32-bit shared-memory integer atomics are native, unlike 64-bit ones.  FP64
// grids reproduce the reference's FP64 weight arithmetic op for op and
// accumulate in FP64.
#include "internal.h"
#include "common.cuh"

#include <math.h>
#include <string.h>
#include <vector>

namespace fg {

constexpr int kTileMax = 16;
constexpr int kMaxPaintGrids = 2;
constexpr double kMaxCellWeight = 8.0 / 27.0;  // largest PCS weight product
constexpr int kMinFixBits = 8;                   // below this: FP32 accumulation

struct AxisParams {
    // FP32 path: x * h - o as double-float (h = Ng/L, o = offset of grid g)
    float h_hi, h_lo;
    float o_hi[kMaxPaintGrids], o_lo[kMaxPaintGrids];
    // FP64 path
    double h;
    double o[kMaxPaintGrids];
};

struct PaintParams {
    AxisParams ax[3];
    int Ng, Ng_pad, nt, ngrids;
    const int *tile_of;   // [Ng]
    const int *start;     // [nt + 1]
};

// ---- per-axis cell coordinate ----------------------------------------------

__device__ __forceinline__ void coord(float x, const AxisParams &a, int g, int Ng, int &b,
                                      float &d) {
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

__device__ __forceinline__ void coord(double x, const AxisParams &a, int g, int Ng, int &b,
                                      double &d) {
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

template <typename P> struct Rec;
template <> struct Rec<float> { using type = float4; };
template <> struct Rec<double> { struct type { double x, y, z; }; };

// ---- 1. key + histogram -------------------------------------------------------

template <typename P>
__global__ void paint_key_kernel(const P *__restrict__ x, const P *__restrict__ y,
                                 const P *__restrict__ z, long Np, PaintParams pp,
                                 uint32_t *__restrict__ key, uint32_t *__restrict__ rank,
                                 uint32_t *__restrict__ hist) {
    const int Ng = pp.Ng, nt = pp.nt;
    for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < Np;
         p += (long)gridDim.x * blockDim.x) {
        const P pos[3] = {x[p], y[p], z[p]};
        int t[3], cls[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            int b0;
            P d;
            coord(pos[a], pp.ax[a], 0, Ng, b0, d);
            const int ta = pp.tile_of[b0];
            const int t0 = pp.start[ta];
            const int te = pp.start[ta + 1] - t0;
            int rmin = b0 - t0, rmax = b0 - t0;
            for (int g = 1; g < pp.ngrids; ++g) {
                int bg;
                P dg;
                coord(pos[a], pp.ax[a], g, Ng, bg, dg);
                const int dl = ((bg - b0 + Ng + 1) % Ng) - 1;  // -1, 0 or +1
                rmin = min(rmin, b0 - t0 + dl);
                rmax = max(rmax, b0 - t0 + dl);
            }
            t[a] = ta;
            cls[a] = nt == 1 ? 0 : (rmin - 1 < 0 ? 1 : (rmax + 2 >= te ? 2 : 0));
        }
        const uint32_t k =
            (uint32_t)((((long)t[0] * nt + t[1]) * nt + t[2]) * 27 + cls[0] * 9 + cls[1] * 3 + cls[2]);
        key[p] = k;
        rank[p] = atomicAdd(&hist[k], 1u);
    }
}

// ---- 2. exclusive scan of the histogram (in place, n + 1 entries) ------------------

constexpr int kScanThreads = 1024;
constexpr int kScanPer = 4;
constexpr int kScanBlock = kScanThreads * kScanPer;

__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t *warp_sums,
                                                         uint32_t *total) {
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
                                     const P *__restrict__ z, long Np,
                                     const uint32_t *__restrict__ key,
                                     const uint32_t *__restrict__ rank,
                                     const uint32_t *__restrict__ off,
                                     typename Rec<P>::type *__restrict__ sorted) {
    for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < Np;
         p += (long)gridDim.x * blockDim.x) {
        const uint32_t dst = off[key[p]] + rank[p];
        typename Rec<P>::type r;
        if constexpr (sizeof(P) == 4) {
            r = make_float4(x[p], y[p], z[p], 0.f);
        } else {
            r.x = x[p];
            r.y = y[p];
            r.z = z[p];
        }
        sorted[dst] = r;
    }
}

// ---- 4. tile paint ---------------------------------------------------------------------

constexpr int kPaintThreads = 256;
constexpr int kMaxSeg = 125;

struct PaintOut {
    void *out[kMaxPaintGrids];
    double scale[kMaxPaintGrids];
    int accumulate[kMaxPaintGrids];
};

template <typename G> struct Acc;
template <> struct Acc<float> { using type = unsigned int; };
template <> struct Acc<double> { using type = double; };

template <typename G>
__global__ void __launch_bounds__(kPaintThreads)
paint_tile_kernel(PaintParams pp, const uint32_t *__restrict__ off,
                  const typename Rec<G>::type *__restrict__ sorted, PaintOut po) {
    using A = typename Acc<G>::type;
    constexpr int T3 = kTileMax * kTileMax * kTileMax;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    A *acc = reinterpret_cast<A *>(smem_raw);  // [ngrids][T3]
    __shared__ uint32_t seg_begin[kMaxSeg];
    __shared__ uint32_t seg_pref[kMaxSeg + 1];
    __shared__ int nseg_s;
    __shared__ int fixbits_s;
    __shared__ int wrapped_s;

    const int Ng = pp.Ng, nt = pp.nt;
    const int tx = blockIdx.x / (nt * nt), ty = (blockIdx.x / nt) % nt, tz = blockIdx.x % nt;
    const int tt[3] = {tx, ty, tz};
    int t0[3], te[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        t0[a] = pp.start[tt[a]];
        te[a] = pp.start[tt[a] + 1] - t0[a];
    }
    const int ngr = pp.ngrids;
    for (int e = threadIdx.x; e < ngr * T3; e += blockDim.x) acc[e] = (A)0;

    if (threadIdx.x == 0) {
        // per axis: list of (neighbour tile, class mask)
        int nopt[3], otile[3][5], ocls[3][5];
        for (int a = 0; a < 3; ++a) {
            int k = 0;
            if (nt == 1) {
                otile[a][k] = tt[a]; ocls[a][k++] = 0;
            } else {
                // own tile: all classes
                for (int c = 0; c < 3; ++c) { otile[a][k] = tt[a]; ocls[a][k++] = c; }
                const int lo = (tt[a] + nt - 1) % nt, hi = (tt[a] + 1) % nt;
                if (nt == 2) {
                    otile[a][k] = hi; ocls[a][k++] = 1;
                    otile[a][k] = hi; ocls[a][k++] = 2;
                } else {
                    otile[a][k] = lo; ocls[a][k++] = 2;  // lower tile, reaching up
                    otile[a][k] = hi; ocls[a][k++] = 1;  // upper tile, reaching down
                }
            }
            nopt[a] = k;
        }
        int ns = 0;
        uint32_t pref = 0;
        for (int i = 0; i < nopt[0]; ++i)
            for (int j = 0; j < nopt[1]; ++j)
                for (int k = 0; k < nopt[2]; ++k) {
                    const long key = (((long)otile[0][i] * nt + otile[1][j]) * nt + otile[2][k]) * 27 +
                                     ocls[0][i] * 9 + ocls[1][j] * 3 + ocls[2][k];
                    const uint32_t b = off[key], e = off[key + 1];
                    if (e > b) {
                        seg_begin[ns] = b;
                        seg_pref[ns] = pref;
                        pref += e - b;
                        ++ns;
                    }
                }
        seg_pref[ns] = pref;
        nseg_s = ns;
        // first try: fixed-point bits for a generous bound on one cell's
        // particle count (four times the mean count of a 4^3 stencil window
        // plus 64); a wrapped cell sum is detected and the tile redone with
        // the bound `pref` (every particle in one cell), which cannot wrap
        const double mean_win = 64.0 * pref / ((double)te[0] * te[1] * te[2]);
        const double cnt = fmin((double)pref, 4.0 * mean_win + 64.0);
        int fb = 31;
        if (pref > 0) fb = (int)floor(log2(4294967295.0 / (cnt * kMaxCellWeight)));
        fixbits_s = fb > 31 ? 31 : fb;
        wrapped_s = 0;
    }
    __syncthreads();
    const int nseg = nseg_s;
    const uint32_t total = seg_pref[nseg];
    int fixbits = fixbits_s;
    bool fixed = fixbits >= kMinFixBits;  // false only for > 5e7 particles in a tile

    for (int attempt = 0; attempt < 2; ++attempt) {
        const float fscale = ldexpf(1.0f, fixbits);
        bool wrapped = false;
        for (uint32_t q = threadIdx.x; q < total; q += blockDim.x) {
            int lo = 0, hi = nseg - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (seg_pref[mid] <= q) lo = mid; else hi = mid - 1;
            }
            const auto r = sorted[seg_begin[lo] + (q - seg_pref[lo])];
            const G pos[3] = {(G)r.x, (G)r.y, (G)r.z};
            for (int g = 0; g < ngr; ++g) {
                int loc[3][4];
                G w[3][4];
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    int b;
                    G d;
                    coord(pos[a], pp.ax[a], g, Ng, b, d);
                    pcs_weights(d, w[a]);
#pragma unroll
                    for (int s = 0; s < 4; ++s) {
                        int c = b - 1 + s;
                        c = c < 0 ? c + Ng : (c >= Ng ? c - Ng : c);
                        const int l = c - t0[a];
                        loc[a][s] = (l >= 0 && l < te[a]) ? l : -1;
                    }
                }
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    if (loc[0][i] < 0) continue;
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        if (loc[1][j] < 0) continue;
                        const G wij = w[0][i] * w[1][j];
                        const int rowb = (loc[0][i] * kTileMax + loc[1][j]) * kTileMax;
#pragma unroll
                        for (int k = 0; k < 4; ++k) {
                            if (loc[2][k] < 0) continue;
                            if constexpr (sizeof(G) == 4) {
                                const float wv = wij * w[2][k];
                                if (fixed) {
                                    const unsigned v = __float2uint_rn(wv * fscale);
                                    const unsigned old = atomicAdd(&acc[g * T3 + rowb + loc[2][k]], v);
                                    wrapped |= (old + v < old);
                                } else {
                                    atomicAdd(reinterpret_cast<float *>(&acc[g * T3 + rowb + loc[2][k]]), wv);
                                }
                            } else {
                                atomicAdd(&acc[g * T3 + rowb + loc[2][k]], __dmul_rn(wij, w[2][k]));
                            }
                        }
                    }
                }
            }
        }
        if (wrapped) wrapped_s = 1;
        __syncthreads();
        const bool redo = wrapped_s && attempt == 0;
        __syncthreads();
        if (!redo) break;
        if (threadIdx.x == 0) wrapped_s = 0;
        // a cell sum wrapped: redo with the bound that cannot wrap
        fixbits = (int)floor(log2(4294967295.0 / ((double)total * kMaxCellWeight)));
        fixbits = fixbits > 31 ? 31 : fixbits;
        fixed = fixbits >= kMinFixBits;
        for (int e = threadIdx.x; e < ngr * T3; e += blockDim.x) acc[e] = (A)0;
        __syncthreads();
    }

    // write the owned cells (and the row padding of the last k tile)
    const bool last_k = (t0[2] + te[2] == Ng);
    const int pad = last_k ? pp.Ng_pad - Ng : 0;
    const int rowlen = te[2] + pad;
    const int ncell = te[0] * te[1] * rowlen;
    for (int g = 0; g < ngr; ++g) {
        G *out = reinterpret_cast<G *>(po.out[g]);
        const G sc = sizeof(G) == 4 ? (G)ldexp(po.scale[g], fixed ? -fixbits : 0) : (G)po.scale[g];
        const int accu = po.accumulate[g];
        for (int e = threadIdx.x; e < ncell; e += blockDim.x) {
            const int lk = e % rowlen, lj = (e / rowlen) % te[1], li = e / (rowlen * te[1]);
            const long gi = ((long)(t0[0] + li) * Ng + (t0[1] + lj)) * pp.Ng_pad + t0[2] + lk;
            G v = 0;
            if (lk < te[2]) {
                const A a = acc[g * T3 + (li * kTileMax + lj) * kTileMax + lk];
                if constexpr (sizeof(G) == 4)
                    v = (fixed ? __uint2float_rn(a) : __uint_as_float(a)) * sc;
                else
                    v = a * sc;
            }
            if (accu) {
                if (lk < te[2]) out[gi] += v;
            } else {
                out[gi] = v;
            }
        }
    }
}

// ---- host side -----------------------------------------------------------------------------

int paint_tiling_create(PaintTiling *t, int Ng, int tile) {
    if (tile > kTileMax || tile < 5) tile = kTileMax;
    int nt = (int)ceil_div(Ng, tile);
    // with more than one tile per axis every extent must be >= 5 so that a
    // stencil reaches at most the adjacent tile and the classes are exclusive
    while (nt > 1 && Ng / nt < 5) --nt;
    std::vector<int> tab(Ng + nt + 1);
    int tmax = 0;
    for (int a = 0; a <= nt; ++a) tab[Ng + a] = (int)((long)a * Ng / nt);
    for (int a = 0; a < nt; ++a) {
        const int s0 = tab[Ng + a], s1 = tab[Ng + a + 1];
        tmax = s1 - s0 > tmax ? s1 - s0 : tmax;
        for (int c = s0; c < s1; ++c) tab[c] = a;
    }
    if (tmax > kTileMax) return set_error(ERR_STATE, "paint tile extent %d > %d", tmax, kTileMax);
    t->Ng = Ng;
    t->nt = nt;
    t->tmax = tmax;
    t->nkeys = (long)nt * nt * nt * 27;
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
    s->bytes = (sizeof(uint32_t) * 2 + 32) * (size_t)s->cap_particles +
               sizeof(uint32_t) * (size_t)s->cap_keys;
    return OK;
}

static void split(double v, float &hi, float &lo) {
    hi = (float)v;
    lo = (float)(v - (double)hi);
}

int paint(const PaintTiling *t, PaintScratch *s, int grid_prec, const void *x, const void *y,
          const void *z, int pos_prec, long Np, double Hinv, const PaintGridSpec *grids,
          int ngrids, cudaStream_t st, cudaEvent_t *ev) {
    if (ngrids < 1 || ngrids > kMaxPaintGrids) return set_error(ERR_ARG, "paint: 1 or 2 grids");
    if (pos_prec != grid_prec)
        return set_error(ERR_ARG, "paint: position precision must match grid precision");
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
    pp.nt = t->nt;
    pp.ngrids = ngrids;
    pp.tile_of = t->d_tables;
    pp.start = t->d_tables + Ng;
    for (int a = 0; a < 3; ++a) {
        split(Hinv, pp.ax[a].h_hi, pp.ax[a].h_lo);
        pp.ax[a].h = Hinv;
        for (int g = 0; g < ngrids; ++g) {
            split(grids[g].offset[a], pp.ax[a].o_hi[g], pp.ax[a].o_lo[g]);
            pp.ax[a].o[g] = grids[g].offset[a];
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
            paint_key_kernel<float><<<gp, 256, 0, st>>>((const float *)x, (const float *)y,
                                                       (const float *)z, Np, pp, s->key, s->rank, s->hist);
        else
            paint_key_kernel<double><<<gp, 256, 0, st>>>((const double *)x, (const double *)y,
                                                        (const double *)z, Np, pp, s->key, s->rank, s->hist);
        FG_LAUNCHED(1);
    }
    if (ev) FG_CUDA(cudaEventRecord(ev[0], st));
    FG_TRY(exclusive_scan(s->hist, t->nkeys + 1, s->scan_tmp, st));
    if (ev) FG_CUDA(cudaEventRecord(ev[1], st));
    if (Np > 0) {
        if (pos_prec == 4)
            paint_scatter_kernel<float><<<gp, 256, 0, st>>>((const float *)x, (const float *)y,
                                                           (const float *)z, Np, s->key, s->rank, s->hist,
                                                           (float4 *)s->sorted);
        else
            paint_scatter_kernel<double><<<gp, 256, 0, st>>>(
                (const double *)x, (const double *)y, (const double *)z, Np, s->key, s->rank, s->hist,
                (Rec<double>::type *)s->sorted);
        FG_LAUNCHED(1);
    }
    if (ev) FG_CUDA(cudaEventRecord(ev[2], st));
    const unsigned ntiles = (unsigned)((long)t->nt * t->nt * t->nt);
    const size_t smem = (size_t)ngrids * kTileMax * kTileMax * kTileMax * (grid_prec == 4 ? 4 : 8);
    if (grid_prec == 4) {
        FG_CUDA(cudaFuncSetAttribute(paint_tile_kernel<float>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        paint_tile_kernel<float><<<ntiles, kPaintThreads, smem, st>>>(pp, s->hist,
                                                                    (const float4 *)s->sorted, po);
    } else {
        FG_CUDA(cudaFuncSetAttribute(paint_tile_kernel<double>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        paint_tile_kernel<double><<<ntiles, kPaintThreads, smem, st>>>(
            pp, s->hist, (const Rec<double>::type *)s->sorted, po);
    }
    FG_LAUNCHED(1);
    if (ev) FG_CUDA(cudaEventRecord(ev[3], st));
    return OK;
}

}  // namespace fg
