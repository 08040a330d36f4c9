// bx_generator.cu -- synthetic cell clusters built on the GPU with BETSE's
// seeding (Cells.make_world, betse/science/cells.py:414-961).
//
// The pipeline, every stage a kernel on the caller's stream:
//   1. the jittered hexagonal seed lattice (_make_cell_lattice,
//      cells.py:742-801): numpy's linspace rows and the legacy
//      np.random.RandomState(seed).rand() jitter, restated bit for bit
//      (MT19937 of Matsumoto & Nishimura, numpy's init_genrand seeding and
//      53-bit doubles);
//   2. pass one: the centroid-Voronoi cell of every lattice point near the
//      disc (Voronoi vertices at triangle centroids, DECMesh(use_centroids=
//      True), math/mesh.py:86) and its area centroid; the centroids inside
//      the disc become the points of
//   3. pass two: the mesh rebuilt on those centroids (clip_and_refine's
//      second pass, mesh.py:2290-2372); its closed cells are the cluster;
//   4. cells ordered along a Z curve of their centres, membranes scaled by
//      scale_cell about the centre and listed as cellVerts lists them
//      (cells.py:978-1175), volumes (cell_vols, :1358-1390), gap-junction
//      partners across each shared Delaunay edge (near_neigh, :1477-1573),
//      the environment grid map (makeECM/environment, :1576-1843) and the
//      cell adjacency.
//
// Delaunay stars without a global triangulation: each point's Voronoi cell
// is the intersection of the half-planes of its bisectors with the points
// of the surrounding buckets, visited ring by ring.  A ring is enough once
// every point not yet visited lies further than twice the cell's furthest
// vertex (the security radius: such a point's bisector cannot cut the cell).
// A cell that keeps an edge of the initial box is unbounded: the point is on
// the convex hull.  The cell's edges, counter-clockwise, are its Delaunay
// neighbours; consecutive neighbours close its triangles.
//
// Floating point follows the restatement in numpy operation by operation:
// products and sums are separate roundings (no contraction), sums of a
// polygon's terms use numpy's pairwise order, triangle centroids add their
// vertices in ascending index order.  hypot and atan2 are CUDA's (within an
// ulp or two of libm's).
#include <cuda_runtime.h>

#include <climits>
#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/bx.h"

void bx_record_error(const char* msg);

namespace {

constexpr int kMaxV = 32;           // vertices of a Voronoi cell while it is clipped
constexpr int kTpb = 128;

// status words raised by the kernels
enum GenFlag { kPolyOverflow = 0, kDuplicate, kFanOrder, kUnpaired, kNFlags };

// ----------------------------------------------------------------- MT19937
constexpr int kMtN = 624, kMtM = 397;
constexpr uint32_t kMatrixA = 0x9908b0dfu, kUpper = 0x80000000u, kLower = 0x7fffffffu;

// n_words tempered outputs of MT19937 seeded by init_genrand(seed), the
// stream numpy's RandomState(seed) draws from.  One CTA of >= 624 threads;
// each twist runs in three phases because words [227, 624) read words
// already twisted in the same pass.
__global__ void k_mt19937(uint32_t seed, int64_t n_words, uint32_t* __restrict__ out) {
  __shared__ uint32_t mt[kMtN];
  const int t = threadIdx.x;
  if (t == 0) {
    uint32_t s = seed;
    for (int i = 0; i < kMtN; ++i) {
      mt[i] = s;
      s = 1812433253u * (s ^ (s >> 30)) + (uint32_t)(i + 1);
    }
  }
  __syncthreads();
  const int lo[3] = {0, kMtN - kMtM, 2 * (kMtN - kMtM)};
  const int hi[3] = {kMtN - kMtM, 2 * (kMtN - kMtM), kMtN};
  for (int64_t base = 0; base < n_words; base += kMtN) {
    for (int ph = 0; ph < 3; ++ph) {
      uint32_t v = 0;
      const bool mine = t >= lo[ph] && t < hi[ph];
      if (mine) {
        const uint32_t nxt = (t == kMtN - 1) ? mt[0] : mt[t + 1];
        const uint32_t y = (mt[t] & kUpper) | (nxt & kLower);
        const uint32_t src = (t < kMtN - kMtM) ? mt[t + kMtM] : mt[t + kMtM - kMtN];
        v = src ^ (y >> 1) ^ ((y & 1u) ? kMatrixA : 0u);
      }
      __syncthreads();
      if (mine) mt[t] = v;
      __syncthreads();
    }
    if (t < kMtN && base + t < n_words) {
      uint32_t y = mt[t];
      y ^= y >> 11;
      y ^= (y << 7) & 0x9d2c5680u;
      y ^= (y << 15) & 0xefc60000u;
      y ^= y >> 18;
      out[base + t] = y;
    }
    __syncthreads();
  }
}

// numpy.linspace(a, b, n)[i]: i * ((b - a) / (n - 1)) + a, the last sample b
__device__ double linspace_at(double a, double b, int n, int i) {
  if (n <= 1) return a;
  if (i == n - 1) return b;
  const double step = __ddiv_rn(__dsub_rn(b, a), (double)(n - 1));
  if (step == 0.0) return __dadd_rn(__dmul_rn(__ddiv_rn((double)i, (double)(n - 1)), __dsub_rn(b, a)), a);
  return __dadd_rn(__dmul_rn((double)i, step), a);
}

__device__ double mt_double(const uint32_t* w, int64_t k) {
  const uint32_t a = w[k] >> 5, b = w[k + 1] >> 6;
  return (a * 67108864.0 + b) / 9007199254740992.0;   // exact: < 2^53 over 2^53
}

// the seed lattice: meshgrid(bx, by) rows then meshgrid(rx, ry) rows,
// x + (disorder*d_cell) * (rand - 0.5), the x draws before the y draws
__global__ void k_lattice(bx_gen_spec sp, const uint32_t* __restrict__ words, double* __restrict__ x,
                          double* __restrict__ y) {
  const int nb = sp.nbx * sp.nby, nr = sp.nrx * sp.nry, N = nb + nr;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  double px, py;
  if (i < nb) {
    px = linspace_at(sp.bx0, sp.bx1, sp.nbx, i % sp.nbx);
    py = linspace_at(sp.by0, sp.by1, sp.nby, i / sp.nbx);
  } else {
    const int j = i - nb;
    px = linspace_at(sp.rx0, sp.rx1, sp.nrx, j % sp.nrx);
    py = linspace_at(sp.ry0, sp.ry1, sp.nry, j / sp.nrx);
  }
  const double ux = mt_double(words, 2 * (int64_t)i);
  const double uy = mt_double(words, 2 * (int64_t)N + 2 * (int64_t)i);
  x[i] = __dadd_rn(px, __dmul_rn(sp.jitter, __dsub_rn(ux, 0.5)));
  y[i] = __dadd_rn(py, __dmul_rn(sp.jitter, __dsub_rn(uy, 0.5)));
}

// min, max and sum of x and y over n points (one CTA; a fixed order)
__global__ void k_bounds(const double* __restrict__ x, const double* __restrict__ y, int n, double* __restrict__ out) {
  __shared__ double s[6][32];
  double v[6] = {INFINITY, -INFINITY, INFINITY, -INFINITY, 0.0, 0.0};
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    v[0] = fmin(v[0], x[i]); v[1] = fmax(v[1], x[i]);
    v[2] = fmin(v[2], y[i]); v[3] = fmax(v[3], y[i]);
    v[4] += x[i]; v[5] += y[i];
  }
  for (int o = 16; o > 0; o >>= 1) {
    v[0] = fmin(v[0], __shfl_xor_sync(0xffffffffu, v[0], o));
    v[1] = fmax(v[1], __shfl_xor_sync(0xffffffffu, v[1], o));
    v[2] = fmin(v[2], __shfl_xor_sync(0xffffffffu, v[2], o));
    v[3] = fmax(v[3], __shfl_xor_sync(0xffffffffu, v[3], o));
    v[4] += __shfl_xor_sync(0xffffffffu, v[4], o);
    v[5] += __shfl_xor_sync(0xffffffffu, v[5], o);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
  if (l == 0)
    for (int k = 0; k < 6; ++k) s[k][w] = v[k];
  __syncthreads();
  if (threadIdx.x == 0) {
    double r[6] = {INFINITY, -INFINITY, INFINITY, -INFINITY, 0.0, 0.0};
    for (int k = 0; k < nw; ++k) {
      r[0] = fmin(r[0], s[0][k]); r[1] = fmax(r[1], s[1][k]);
      r[2] = fmin(r[2], s[2][k]); r[3] = fmax(r[3], s[3][k]);
      r[4] += s[4][k]; r[5] += s[5][k];
    }
    for (int k = 0; k < 6; ++k) out[k] = r[k];
  }
}

// ------------------------------------------------------------ scan and sort
// exclusive prefix sum of 1024-element blocks; block totals to sums
__global__ void k_scan_block(const int* __restrict__ in, int* __restrict__ out, int* __restrict__ sums, int n) {
  __shared__ int wt[32];
  const int i = blockIdx.x * 1024 + threadIdx.x;
  const int v = i < n ? in[i] : 0;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const int u = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += u;
  }
  if (lane == 31) wt[w] = x;
  __syncthreads();
  if (w == 0) {
    int t = wt[lane];
    for (int o = 1; o < 32; o <<= 1) {
      const int u = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += u;
    }
    wt[lane] = t;
  }
  __syncthreads();
  const int ex = x - v + (w ? wt[w - 1] : 0);
  if (i < n) out[i] = ex;
  if (threadIdx.x == 1023) sums[blockIdx.x] = ex + v;
}

__global__ void k_scan_add(int* __restrict__ out, const int* __restrict__ offs, int n) {
  const int i = blockIdx.x * 1024 + threadIdx.x;
  if (i < n) out[i] += offs[blockIdx.x];
}

constexpr int kRsThreads = 256, kRsItems = 4, kRsTile = kRsThreads * kRsItems;

__global__ void k_rs_hist(const uint32_t* __restrict__ keys, int n, int shift, int* __restrict__ hist, int nblk) {
  __shared__ int h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  for (int k = 0; k < kRsItems; ++k) {
    const int i = blockIdx.x * kRsTile + k * kRsThreads + threadIdx.x;
    if (i < n) atomicAdd(&h[(keys[i] >> shift) & 255u], 1);
  }
  __syncthreads();
  hist[threadIdx.x * nblk + blockIdx.x] = h[threadIdx.x];
}

// stable scatter: a tile's elements in order, chunk by chunk; within a
// chunk, warps in order and lanes in order (rank among equal digits)
__global__ void k_rs_scatter(const uint32_t* __restrict__ keys, const int* __restrict__ vals,
                             uint32_t* __restrict__ keys_out, int* __restrict__ vals_out, int n, int shift,
                             const int* __restrict__ offs, int nblk) {
  __shared__ int base[256];
  __shared__ int wcnt[kRsThreads / 32][257];
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  base[t] = offs[t * nblk + blockIdx.x];
  for (int k = 0; k < kRsItems; ++k) {
    for (int j = t; j < (kRsThreads / 32) * 257; j += kRsThreads) (&wcnt[0][0])[j] = 0;
    __syncthreads();
    const int i = blockIdx.x * kRsTile + k * kRsThreads + t;
    const bool valid = i < n;
    const uint32_t key = valid ? keys[i] : 0u;
    const int d = valid ? (int)((key >> shift) & 255u) : 256;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const int rank = __popc(peers & ((1u << lane) - 1u));
    if (rank == 0) wcnt[w][d] = __popc(peers);
    __syncthreads();
    if (valid) {
      int pre = 0;
      for (int ww = 0; ww < w; ++ww) pre += wcnt[ww][d];
      const int pos = base[d] + pre + rank;
      keys_out[pos] = key;
      vals_out[pos] = vals[i];
    }
    __syncthreads();
    int tot = 0;
    for (int ww = 0; ww < kRsThreads / 32; ++ww) tot += wcnt[ww][t];
    base[t] += tot;
    __syncthreads();
  }
}

__global__ void k_iota(int* __restrict__ v, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) v[i] = i;
}

// ------------------------------------------------------------ host helpers
struct DevBuf {
  std::vector<void*> ptrs;
  ~DevBuf() {
    for (void* p : ptrs) cudaFree(p);
  }
  template <class T>
  T* get(size_t n) {
    void* p = nullptr;
    if (cudaMalloc(&p, (n ? n : 1) * sizeof(T)) != cudaSuccess) return nullptr;
    ptrs.push_back(p);
    return static_cast<T*>(p);
  }
};

struct GenError {
  int code;
  std::string msg;
};

#define GEN_CHECK(expr, what)                                                     \
  do {                                                                            \
    cudaError_t e_ = (expr);                                                      \
    if (e_ != cudaSuccess) throw GenError{BX_ECUDA, std::string(what) + ": " + cudaGetErrorString(e_)}; \
  } while (0)

template <class T>
T* need(DevBuf& b, size_t n, const char* what) {
  T* p = b.get<T>(n);
  if (!p) throw GenError{BX_ENOMEM, std::string("bx_generate_cluster: cannot allocate ") + what};
  return p;
}

inline int nblocks(int64_t n, int tpb) { return (int)((n + tpb - 1) / tpb); }

// exclusive scan of n ints (in may equal out); returns nothing, total = out[n-1] + in[n-1]
void scan_excl(DevBuf& b, const int* in, int* out, int n, cudaStream_t s) {
  if (n <= 0) return;
  const int nb = nblocks(n, 1024);
  int* sums = need<int>(b, nb, "scan");
  k_scan_block<<<nb, 1024, 0, s>>>(in, out, sums, n);
  if (nb > 1) {
    int* so = need<int>(b, nb, "scan");
    scan_excl(b, sums, so, nb, s);
    k_scan_add<<<nb, 1024, 0, s>>>(out, so, n);
  }
  GEN_CHECK(cudaGetLastError(), "scan");
}

// stable LSD radix sort of (key, value) pairs on the low key_bits bits;
// the sorted pairs end in keys/vals
void radix_sort(DevBuf& b, uint32_t* keys, int* vals, int n, int key_bits, cudaStream_t s) {
  if (n <= 1) return;
  const int nblk = nblocks(n, kRsTile);
  uint32_t* k2 = need<uint32_t>(b, n, "sort keys");
  int* v2 = need<int>(b, n, "sort values");
  int* hist = need<int>(b, (size_t)256 * nblk, "sort histogram");
  uint32_t* ka = keys; int* va = vals;
  uint32_t* kb = k2; int* vb = v2;
  for (int shift = 0; shift < key_bits; shift += 8) {
    k_rs_hist<<<nblk, kRsThreads, 0, s>>>(ka, n, shift, hist, nblk);
    scan_excl(b, hist, hist, 256 * nblk, s);
    k_rs_scatter<<<nblk, kRsThreads, 0, s>>>(ka, va, kb, vb, n, shift, hist, nblk);
    GEN_CHECK(cudaGetLastError(), "radix sort");
    std::swap(ka, kb);
    std::swap(va, vb);
  }
  if (ka != keys) {
    GEN_CHECK(cudaMemcpyAsync(keys, ka, (size_t)n * 4, cudaMemcpyDeviceToDevice, s), "radix sort");
    GEN_CHECK(cudaMemcpyAsync(vals, va, (size_t)n * 4, cudaMemcpyDeviceToDevice, s), "radix sort");
  }
}

// ------------------------------------------------------------ bucket grid
struct Grid {
  double x0, y0, h;
  int nx, ny;
  const int* start;   // [nx*ny] first sorted slot of the bucket
  const int* end;     // [nx*ny] one past its last slot
  const int* idx;     // [n] point index per sorted slot
  const double* px;
  const double* py;
  int n;              // points
};

__device__ int bucket_of(double v, double v0, double h, int n) {
  int b = (int)floor((v - v0) / h);
  return b < 0 ? 0 : (b >= n ? n - 1 : b);
}

__global__ void k_bucket_keys(const double* __restrict__ x, const double* __restrict__ y, int n, double x0, double y0,
                              double h, int nx, int ny, uint32_t* __restrict__ key) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  key[i] = (uint32_t)(bucket_of(y[i], y0, h, ny) * nx + bucket_of(x[i], x0, h, nx));
}

__global__ void k_bucket_ranges(const uint32_t* __restrict__ key, int n, int* __restrict__ start, int* __restrict__ end) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t k = key[i];
  if (i == 0 || key[i - 1] != k) start[k] = i;
  if (i == n - 1 || key[i + 1] != k) end[k] = i + 1;
}

// ------------------------------------------------------------ Voronoi stars
// The cell is kept relative to its point: vertices (vx, vy), and lab[a] the
// label of the edge from vertex a to vertex a+1 (the neighbour across it;
// -1 for an edge of the initial box).

// Clip the cell by the bisector of the point and a candidate at offset
// (dx, dy), label iq: keep x with (x . d) <= |d|^2 / 2.  Returns the new
// vertex count (unchanged when the bisector misses the cell), -1 when the
// cell would exceed kMaxV vertices; r2max becomes the furthest vertex.
__device__ int clip_cell(double* vx, double* vy, int* lab, int n, double dx, double dy, double d2, int iq,
                         double* r2max) {
  double f[kMaxV];
  const double c = 0.5 * d2;
  bool out_any = false;
  for (int a = 0; a < n; ++a) {
    f[a] = vx[a] * dx + vy[a] * dy - c;
    out_any |= f[a] > 0.0;
  }
  if (!out_any) return n;
  double ox[kMaxV], oy[kMaxV];
  int ol[kMaxV];
  int m = 0;
  for (int a = 0; a < n; ++a) {
    const int e = (a + 1 == n) ? 0 : a + 1;
    if (f[a] <= 0.0) {
      if (m >= kMaxV) return -1;
      ox[m] = vx[a]; oy[m] = vy[a]; ol[m] = lab[a]; ++m;
      if (f[e] > 0.0) {
        if (m >= kMaxV) return -1;
        const double t = f[a] / (f[a] - f[e]);
        ox[m] = vx[a] + t * (vx[e] - vx[a]); oy[m] = vy[a] + t * (vy[e] - vy[a]); ol[m] = iq; ++m;
      }
    } else if (f[e] <= 0.0) {
      if (m >= kMaxV) return -1;
      const double t = f[a] / (f[a] - f[e]);
      ox[m] = vx[a] + t * (vx[e] - vx[a]); oy[m] = vy[a] + t * (vy[e] - vy[a]); ol[m] = lab[a]; ++m;
    }
  }
  double r2 = 0.0;
  for (int a = 0; a < m; ++a) {
    vx[a] = ox[a]; vy[a] = oy[a]; lab[a] = ol[a];
    r2 = fmax(r2, vx[a] * vx[a] + vy[a] * vy[a]);
  }
  *r2max = r2;
  return m;
}

// The Delaunay neighbours of point query[q] (or q), counter-clockwise, as
// the labels of its cell's edges (-1: an unbounded cell, the point is on the
// convex hull).  The buckets are visited ring by ring, up to ring kRings; a
// cell not settled by then (at the hull, or next to a sliver triangle whose
// circumcentre is far away) is saved and its query listed for k_star_scan.
constexpr int kRings = 4;

struct SlowCells {
  int* list;       // queries handed over
  int* count;
  double* vx;      // [nq][kMaxV] the cell so far
  double* vy;
  int* lab;
  int* n;          // [nq]
};

__global__ void __launch_bounds__(kTpb) k_star(Grid g, const int* __restrict__ query, int nq, int* __restrict__ nbr,
                                               int* __restrict__ nnb, int* __restrict__ flags, SlowCells slow) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq) return;
  const int ip = query ? query[q] : q;
  const double px = g.px[ip], py = g.py[ip];
  double vx[kMaxV], vy[kMaxV];
  int lab[kMaxV];
  // the initial box: far enough that a bounded cell's furthest vertex (the
  // circumcentre of a sliver triangle at the hull) still lies inside it
  const double B = 1e4 * g.h * (double)(g.nx + g.ny + 4);
  vx[0] = -B; vy[0] = -B; vx[1] = B; vy[1] = -B; vx[2] = B; vy[2] = B; vx[3] = -B; vy[3] = B;
  lab[0] = lab[1] = lab[2] = lab[3] = -1;
  int n = 4;
  double r2max = 2.0 * B * B;
  bool settled = false;
  const int bi = bucket_of(px, g.x0, g.h, g.nx), bj = bucket_of(py, g.y0, g.h, g.ny);
  for (int k = 0; k <= kRings && n > 0; ++k) {
    // the buckets at Chebyshev distance k from (bi, bj)
    for (int dj = -k; dj <= k && n > 0; ++dj) {
      const int j = bj + dj;
      if (j < 0 || j >= g.ny) continue;
      const int step = (dj == -k || dj == k) ? 1 : 2 * k;
      for (int di = -k; di <= k && n > 0; di += (step ? step : 1)) {
        const int i = bi + di;
        if (i < 0 || i >= g.nx) continue;
        const int b = j * g.nx + i;
        for (int sidx = g.start[b]; sidx < g.end[b] && n > 0; ++sidx) {
          const int iq = g.idx[sidx];
          if (iq == ip) continue;
          const double dx = g.px[iq] - px, dy = g.py[iq] - py;
          const double d2 = dx * dx + dy * dy;
          if (d2 == 0.0) { atomicAdd(flags + kDuplicate, 1); continue; }
          if (0.25 * d2 >= r2max) continue;
          n = clip_cell(vx, vy, lab, n, dx, dy, d2, iq, &r2max);
        }
      }
    }
    if (n <= 0) break;
    // security radius of the buckets visited so far
    const bool lx = bi - k <= 0, hx = bi + k >= g.nx - 1, ly = bj - k <= 0, hy = bj + k >= g.ny - 1;
    if (lx && hx && ly && hy) { settled = true; break; }     // every point visited
    double rs = INFINITY;
    if (!lx) rs = fmin(rs, px - (g.x0 + (double)(bi - k) * g.h));
    if (!hx) rs = fmin(rs, (g.x0 + (double)(bi + k + 1) * g.h) - px);
    if (!ly) rs = fmin(rs, py - (g.y0 + (double)(bj - k) * g.h));
    if (!hy) rs = fmin(rs, (g.y0 + (double)(bj + k + 1) * g.h) - py);
    if (4.0 * r2max < rs * rs) { settled = true; break; }
  }
  if (n <= 0) {
    atomicAdd(flags + kPolyOverflow, 1);
    nnb[q] = 0;
    return;
  }
  if (!settled) {
    const int at = atomicAdd(slow.count, 1);
    slow.list[at] = q;
    slow.n[q] = n;
    for (int a = 0; a < n; ++a) {
      slow.vx[(int64_t)q * kMaxV + a] = vx[a];
      slow.vy[(int64_t)q * kMaxV + a] = vy[a];
      slow.lab[(int64_t)q * kMaxV + a] = lab[a];
    }
    return;
  }
  nnb[q] = n;
  for (int a = 0; a < n; ++a) nbr[(int64_t)q * kMaxV + a] = lab[a];
}

// One CTA per cell handed over by k_star: every point of the set is tested
// against the cell in parallel; those whose bisector cuts it (a superset of
// the missing neighbours: the cell only shrinks) are collected, then clipped
// nearest first in rounds.
constexpr int kScanThreads = 256, kScanCand = 2048;

__global__ void __launch_bounds__(kScanThreads) k_star_scan(const double* __restrict__ X, const double* __restrict__ Y,
                                                            int npts, const int* __restrict__ query, SlowCells slow,
                                                            int* __restrict__ nbr, int* __restrict__ nnb,
                                                            int* __restrict__ flags) {
  __shared__ double svx[kMaxV], svy[kMaxV];
  __shared__ float fvx[kMaxV], fvy[kMaxV];
  __shared__ int slab[kMaxV];
  __shared__ int cand[kScanCand];
  __shared__ double cd2[kScanCand];
  __shared__ int ncand;
  const int q = slow.list[blockIdx.x];
  const int ip = query ? query[q] : q;
  const double px = X[ip], py = Y[ip];
  const int n0 = slow.n[q];
  for (int a = threadIdx.x; a < n0; a += blockDim.x) {
    svx[a] = slow.vx[(int64_t)q * kMaxV + a];
    svy[a] = slow.vy[(int64_t)q * kMaxV + a];
    fvx[a] = (float)svx[a];
    fvy[a] = (float)svy[a];
    slab[a] = slow.lab[(int64_t)q * kMaxV + a];
  }
  if (threadIdx.x == 0) ncand = 0;
  __syncthreads();
  for (int i = threadIdx.x; i < npts; i += blockDim.x) {
    if (i == ip) continue;
    const double dx = X[i] - px, dy = Y[i] - py;
    const double d2 = dx * dx + dy * dy;
    if (d2 == 0.0) continue;
    // the cut test in FP32 first: with g = v.d - c, |g32 - g| stays below
    // 1e-6 (|vx dx| + |vy dy| + c) (conversions and products round to 2^-24
    // each), so only a vertex within that margin of the threshold needs FP64
    const double c = 0.5 * d2;
    const float fdx = (float)dx, fdy = (float)dy, fc = (float)c;
    const float thr = fc * 1e-12f;
    bool cut = false;
    for (int a = 0; a < n0 && !cut; ++a) {
      const float gx = fvx[a] * fdx, gy = fvy[a] * fdy;
      const float g = gx + gy - fc;
      const float err = (fabsf(gx) + fabsf(gy) + fc) * 1e-6f;
      if (g > thr + err) cut = true;
      else if (g >= -err) cut = svx[a] * dx + svy[a] * dy - c > 1e-12 * c;
    }
    if (!cut) continue;
    bool known = false;                 // already a neighbour: its bisector holds an edge
    for (int a = 0; a < n0; ++a) known |= slab[a] == i;
    if (known) continue;
    const int at = atomicAdd(&ncand, 1);
    if (at < kScanCand) { cand[at] = i; cd2[at] = d2; }
  }
  __syncthreads();
  const int nc = ncand;
  if (nc > kScanCand) {
    if (threadIdx.x == 0) {
      atomicAdd(flags + kPolyOverflow, 1);
      nnb[q] = 0;
    }
    return;
  }
  // Rounds: every thread finds, among its candidates, the nearest one (ties
  // by index) whose bisector still cuts the cell; the block's nearest is
  // clipped by thread 0.  The cell only shrinks, so a candidate that stops
  // cutting never cuts again; the rounds end when none cuts (about as many
  // rounds as the cell has edges).
  __shared__ int sn;
  __shared__ double sr2;
  __shared__ double bd2[kScanThreads / 32];
  __shared__ int bix[kScanThreads / 32];
  if (threadIdx.x == 0) {
    sn = n0;
    double r2 = 0.0;
    for (int a = 0; a < n0; ++a) r2 = fmax(r2, svx[a] * svx[a] + svy[a] * svy[a]);
    sr2 = r2;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int round = 0; round <= nc; ++round) {
    const int n = sn;
    const double r2max = sr2;
    double best = INFINITY;
    int bi = INT_MAX;
    for (int j = threadIdx.x; j < nc; j += blockDim.x) {
      const double d2 = cd2[j];
      if (0.25 * d2 >= r2max || cand[j] < 0) continue;
      const double dx = X[cand[j]] - px, dy = Y[cand[j]] - py;
      const double c = 0.5 * d2;
      bool cut = false;
      for (int a = 0; a < n && !cut; ++a) cut = svx[a] * dx + svy[a] * dy - c > 0.0;
      if (!cut) { cand[j] = -1; continue; }       // never cuts again
      if (d2 < best || (d2 == best && cand[j] < bi)) { best = d2; bi = cand[j]; }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const double ob = __shfl_down_sync(0xffffffffu, best, o);
      const int oi = __shfl_down_sync(0xffffffffu, bi, o);
      if (ob < best || (ob == best && oi < bi)) { best = ob; bi = oi; }
    }
    if (lane == 0) { bd2[wid] = best; bix[wid] = bi; }
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
        if (bd2[w] < best || (bd2[w] == best && bix[w] < bi)) { best = bd2[w]; bi = bix[w]; }
      if (bi == INT_MAX) {
        sn = -sn - 1;                                  // done (the count, encoded)
      } else {
        double r2 = r2max;
        const int m = clip_cell(svx, svy, slab, n, X[bi] - px, Y[bi] - py, best, bi, &r2);
        sn = m;
        sr2 = r2;
        for (int j = 0; j < nc; ++j)
          if (cand[j] == bi) { cand[j] = -1; break; }
      }
    }
    __syncthreads();
    if (sn <= 0) break;
  }
  if (threadIdx.x != 0) return;
  const int n = sn < 0 ? -sn - 1 : sn;
  if (sn == 0 || n <= 0) {
    atomicAdd(flags + kPolyOverflow, 1);
    nnb[q] = 0;
    return;
  }
  nnb[q] = n;
  for (int a = 0; a < n; ++a) nbr[(int64_t)q * kMaxV + a] = slab[a];
}

// numpy's float64 sum of a short contiguous array (pairwise_sum: a plain
// loop below 8 terms, eight interleaved accumulators up to 128)
__device__ double np_sum(const double* a, int n) {
  if (n < 8) {
    double r = 0.0;
    for (int i = 0; i < n; ++i) r = __dadd_rn(r, a[i]);
    return r;
  }
  double r[8];
  for (int j = 0; j < 8; ++j) r[j] = a[j];
  int i = 8;
  for (; i < n - (n % 8); i += 8)
    for (int j = 0; j < 8; ++j) r[j] = __dadd_rn(r[j], a[i + j]);
  double res = __dadd_rn(__dadd_rn(__dadd_rn(r[0], r[1]), __dadd_rn(r[2], r[3])),
                         __dadd_rn(__dadd_rn(r[4], r[5]), __dadd_rn(r[6], r[7])));
  for (; i < n; ++i) res = __dadd_rn(res, a[i]);
  return res;
}

// area centroid of a polygon (DECMesh.poly_centroid): with Q the vertices
// rolled by one, a = Px Qy - Qx Py, A = sum(a) / 2,
// c = (sum((Px + Qx) a), sum((Py + Qy) a)) / (6 A)
__device__ void poly_centroid(const double* X, const double* Y, int n, double* cx, double* cy) {
  double a[kMaxV], sx[kMaxV], sy[kMaxV];
  for (int k = 0; k < n; ++k) {
    const int e = (k + 1 == n) ? 0 : k + 1;
    a[k] = __dsub_rn(__dmul_rn(X[k], Y[e]), __dmul_rn(X[e], Y[k]));
  }
  for (int k = 0; k < n; ++k) {
    const int e = (k + 1 == n) ? 0 : k + 1;
    sx[k] = __dmul_rn(__dadd_rn(X[k], X[e]), a[k]);
    sy[k] = __dmul_rn(__dadd_rn(Y[k], Y[e]), a[k]);
  }
  const double A = __ddiv_rn(np_sum(a, n), 2.0);
  const double d = __dmul_rn(6.0, A);
  *cx = __ddiv_rn(np_sum(sx, n), d);
  *cy = __ddiv_rn(np_sum(sy, n), d);
}

// The closed fan of a point: its triangles (point, nb[i], nb[i+1]) in the
// order of their centroids' angles about the point (atan2 from -pi), the
// centroids as the polygon's vertices, and per polygon edge k (from vertex
// k-1 to vertex k) the neighbour across it.  Returns the vertex count, 0 for
// a hull point (an unbounded Voronoi cell) or a fan of fewer than 3.
__device__ int closed_fan(int ip, const double* __restrict__ X, const double* __restrict__ Y, const int* lab, int n,
                          double* VX, double* VY, int* other, int* flags) {
  if (n < 3) return 0;
  for (int i = 0; i < n; ++i)
    if (lab[i] < 0) return 0;
  double tx[kMaxV], ty[kMaxV], ang[kMaxV];
  const double px = X[ip], py = Y[ip];
  int r = 0;
  for (int i = 0; i < n; ++i) {
    int a = ip, b = lab[i], c = lab[(i + 1 == n) ? 0 : i + 1];
    // centroid of the triangle: vertices added in ascending index order
    if (a > b) { const int t = a; a = b; b = t; }
    if (b > c) { const int t = b; b = c; c = t; }
    if (a > b) { const int t = a; a = b; b = t; }
    tx[i] = __ddiv_rn(__dadd_rn(__dadd_rn(X[a], X[b]), X[c]), 3.0);
    ty[i] = __ddiv_rn(__dadd_rn(__dadd_rn(Y[a], Y[b]), Y[c]), 3.0);
    ang[i] = atan2(__dsub_rn(ty[i], py), __dsub_rn(tx[i], px));
    if (ang[i] < ang[r]) r = i;
  }
  for (int k = 0; k < n; ++k) {
    const int i = (r + k) % n;
    VX[k] = tx[i];
    VY[k] = ty[i];
    other[k] = lab[i];
    if (k && !(ang[i] > ang[(r + k - 1) % n])) atomicAdd(flags + kFanOrder, 1);
  }
  return n;
}

// pass one: the area centroid of each queried lattice point's closed cell;
// keep[q] = 1 when it lies inside the disc
__global__ void __launch_bounds__(kTpb) k_pass1(const double* __restrict__ X, const double* __restrict__ Y,
                                                const int* __restrict__ query, int nq, const int* __restrict__ nbr,
                                                const int* __restrict__ nnb, double cx0, double cy0, double radius,
                                                double* __restrict__ c0x, double* __restrict__ c0y,
                                                int* __restrict__ keep, int* __restrict__ flags) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq) return;
  double VX[kMaxV], VY[kMaxV];
  int other[kMaxV];
  const int n = closed_fan(query[q], X, Y, nbr + (int64_t)q * kMaxV, nnb[q], VX, VY, other, flags);
  int k = 0;
  if (n) {
    double cx, cy;
    poly_centroid(VX, VY, n, &cx, &cy);
    c0x[q] = cx;
    c0y[q] = cy;
    k = hypot(__dsub_rn(cx, cx0), __dsub_rn(cy, cy0)) < radius;
  }
  keep[q] = k;
}

// pass two: each point's closed cell (vertices, neighbours across its
// edges, area centroid); keep[q] = 1 for a closed cell
__global__ void __launch_bounds__(kTpb) k_pass2(const double* __restrict__ X, const double* __restrict__ Y, int nq,
                                                const int* __restrict__ nbr, const int* __restrict__ nnb,
                                                double* __restrict__ PX, double* __restrict__ PY,
                                                int* __restrict__ other, int* __restrict__ nv,
                                                double* __restrict__ pcx, double* __restrict__ pcy,
                                                int* __restrict__ keep, int* __restrict__ flags) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq) return;
  double VX[kMaxV], VY[kMaxV];
  int ot[kMaxV];
  const int n = closed_fan(q, X, Y, nbr + (int64_t)q * kMaxV, nnb[q], VX, VY, ot, flags);
  nv[q] = n;
  keep[q] = n > 0;
  if (!n) return;
  for (int k = 0; k < n; ++k) {
    PX[(int64_t)q * kMaxV + k] = VX[k];
    PY[(int64_t)q * kMaxV + k] = VY[k];
    other[(int64_t)q * kMaxV + k] = ot[k];
  }
  double cx, cy;
  poly_centroid(VX, VY, n, &cx, &cy);
  pcx[q] = cx;
  pcy[q] = cy;
}

// stream compaction by a 0/1 flag after its exclusive scan
__global__ void k_compact(const int* __restrict__ flag, const int* __restrict__ pos, int n, const int* __restrict__ src,
                          int* __restrict__ dst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && flag[i]) dst[pos[i]] = src ? src[i] : i;
}

__global__ void k_gather2(const int* __restrict__ idx, int n, const double* __restrict__ ax,
                          const double* __restrict__ ay, double* __restrict__ bx, double* __restrict__ by) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) { bx[i] = ax[idx[i]]; by[i] = ay[idx[i]]; }
}

// lattice points within `reach` of the centre
__global__ void k_near_disc(const double* __restrict__ x, const double* __restrict__ y, int n, double cx, double cy,
                            double reach, int* __restrict__ flag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) flag[i] = hypot(x[i] - cx, y[i] - cy) < reach;
}

// Z-curve key of each kept cell's centre (16 bits per axis, as
// ((c - lo) / span * 65535) truncated; bit b of x at 2b, of y at 2b+1)
__global__ void k_zkeys(const int* __restrict__ seeds, int C, const double* __restrict__ pcx,
                        const double* __restrict__ pcy, const double* __restrict__ bnd, uint32_t* __restrict__ key) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= C) return;
  const int s = seeds[c];
  const double lox = bnd[0], loy = bnd[2];
  const double spx = fmax(__dsub_rn(bnd[1], lox), 1e-30), spy = fmax(__dsub_rn(bnd[3], loy), 1e-30);
  const uint32_t qx = (uint32_t)__dmul_rn(__ddiv_rn(__dsub_rn(pcx[s], lox), spx), 65535.0);
  const uint32_t qy = (uint32_t)__dmul_rn(__ddiv_rn(__dsub_rn(pcy[s], loy), spy), 65535.0);
  uint32_t k = 0;
  for (int b = 0; b < 16; ++b) k |= (((qx >> b) & 1u) << (2 * b)) | (((qy >> b) & 1u) << (2 * b + 1));
  key[c] = k;
}

__global__ void k_gather_centres(const int* __restrict__ seeds, int C, const double* __restrict__ pcx,
                                 const double* __restrict__ pcy, double* __restrict__ x, double* __restrict__ y) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < C) { x[c] = pcx[seeds[c]]; y[c] = pcy[seeds[c]]; }
}

__global__ void k_cell_counts(const int* __restrict__ cell_seed, int C, const int* __restrict__ nv,
                              int* __restrict__ counts, int* __restrict__ seed_to_cell) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= C) return;
  counts[c] = nv[cell_seed[c]];
  seed_to_cell[cell_seed[c]] = c;
}

// Membranes of each cell (cellVerts, cell_vols): vertices scaled toward the
// centre, V = scale (V - c) + c; membrane k joins vertex k-1 and vertex k;
// mid, unit normal (ty, -tx), area = length * height, R_rads, volume
// sum of 0.5 R sa in membrane order, cell area sum of sa.
__global__ void k_membranes(const int* __restrict__ cell_seed, int C, const int* __restrict__ ptr,
                            const double* __restrict__ PX, const double* __restrict__ PY,
                            const int* __restrict__ other, const double* __restrict__ pcx,
                            const double* __restrict__ pcy, double scale, double height,
                            double* __restrict__ mid_x, double* __restrict__ mid_y, double* __restrict__ nx,
                            double* __restrict__ ny, double* __restrict__ sa, double* __restrict__ rr,
                            int* __restrict__ oth, int* __restrict__ m2c, double* __restrict__ vol,
                            double* __restrict__ csa, double* __restrict__ divi) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= C) return;
  const int s = cell_seed[c];
  const int m0 = ptr[c], d = ptr[c + 1] - m0;
  const double cx = pcx[s], cy = pcy[s];
  const double* X = PX + (int64_t)s * kMaxV;
  const double* Y = PY + (int64_t)s * kMaxV;
  double v = 0.0, a = 0.0;
  double qx = __dadd_rn(__dmul_rn(scale, __dsub_rn(X[d - 1], cx)), cx);
  double qy = __dadd_rn(__dmul_rn(scale, __dsub_rn(Y[d - 1], cy)), cy);
  for (int k = 0; k < d; ++k) {
    const double px2 = __dadd_rn(__dmul_rn(scale, __dsub_rn(X[k], cx)), cx);
    const double py2 = __dadd_rn(__dmul_rn(scale, __dsub_rn(Y[k], cy)), cy);
    const double mx = __ddiv_rn(__dadd_rn(qx, px2), 2.0), my = __ddiv_rn(__dadd_rn(qy, py2), 2.0);
    const double tx = __dsub_rn(px2, qx), ty = __dsub_rn(py2, qy);
    const double len = hypot(tx, ty);
    const double ux = __ddiv_rn(tx, len), uy = __ddiv_rn(ty, len);
    const double area = __dmul_rn(len, height);
    const double R = hypot(__dsub_rn(mx, cx), __dsub_rn(my, cy));
    const int m = m0 + k;
    mid_x[m] = mx; mid_y[m] = my;
    nx[m] = uy; ny[m] = -ux;
    sa[m] = area;
    rr[m] = R;
    oth[m] = other[(int64_t)s * kMaxV + k];
    m2c[m] = c;
    v = __dadd_rn(v, __dmul_rn(__dmul_rn(0.5, R), area));
    a = __dadd_rn(a, area);
    qx = px2; qy = py2;
  }
  vol[c] = v;
  csa[c] = a;
  divi[c] = __ddiv_rn(v, a);
}

// the partner of membrane m across its Delaunay edge: the membrane of the
// neighbour's cell whose own neighbour is m's cell's seed; a neighbour that
// is not a cell of the cluster leaves m a boundary membrane (partner m)
__global__ void k_pair(int M, const int* __restrict__ m2c, const int* __restrict__ oth,
                       const int* __restrict__ cell_seed, const int* __restrict__ seed_to_cell,
                       const int* __restrict__ ptr, int* __restrict__ nn, int* __restrict__ flags) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= M) return;
  const int c2 = seed_to_cell[oth[m]];
  int r = m;
  if (c2 >= 0) {
    const int s = cell_seed[m2c[m]];
    r = -1;
    for (int k = ptr[c2]; k < ptr[c2 + 1]; ++k)
      if (oth[k] == s) { r = k; break; }
    if (r < 0) { atomicAdd(flags + kUnpaired, 1); r = m; }
  }
  nn[m] = r;
}

// grid centres: cx[i] = (xv[i] + xv[i+1]) / 2 with xv = linspace(lo, hi, n + 1)
__global__ void k_grid_centres(double lo, double hi, int n, double* __restrict__ c) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) c[i] = __ddiv_rn(__dadd_rn(linspace_at(lo, hi, n + 1, i), linspace_at(lo, hi, n + 1, i + 1)), 2.0);
}

// nearest grid centre per axis (searchsorted left, clipped to [1, n-1], then
// the lower neighbour on a tie): map_mem2ecm = iy * nx + jx
__device__ int nearest_centre(const double* c, int n, double v) {
  int lo = 0, hi = n;                 // first i with c[i] >= v
  while (lo < hi) {
    const int md = (lo + hi) >> 1;
    if (c[md] < v) lo = md + 1; else hi = md;
  }
  int j = lo < 1 ? 1 : (lo > n - 1 ? n - 1 : lo);
  if (fabs(c[j - 1] - v) <= fabs(c[j] - v)) j -= 1;
  return j;
}

__global__ void k_grid_map(int M, const double* __restrict__ mx, const double* __restrict__ my,
                          const double* __restrict__ cx, int gnx, const double* __restrict__ cy, int gny,
                          int* __restrict__ map, uint32_t* __restrict__ key, int* __restrict__ val) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= M) return;
  const int g = nearest_centre(cy, gny, my[m]) * gnx + nearest_centre(cx, gnx, mx[m]);
  map[m] = g;
  key[m] = (uint32_t)g;
  val[m] = m;
}

// membrane area per grid cell, summed in membrane order (np.bincount)
__global__ void k_grid_area(int M, const uint32_t* __restrict__ key, const int* __restrict__ mem,
                          const double* __restrict__ sa, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= M || (i > 0 && key[i - 1] == key[i])) return;
  double s = 0.0;
  for (int k = i; k < M && key[k] == key[i]; ++k) s = __dadd_rn(s, sa[mem[k]]);
  out[key[i]] = s;
}

__global__ void k_nn_counts(int C, const int* __restrict__ ptr, const int* __restrict__ nn, int* __restrict__ cnt) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= C) return;
  int k = 0;
  for (int m = ptr[c]; m < ptr[c + 1]; ++m) k += nn[m] != m;
  cnt[c] = k;
}

// each cell's neighbouring cells in ascending order
__global__ void k_nn_fill(int C, const int* __restrict__ ptr, const int* __restrict__ nn, const int* __restrict__ m2c,
                          const int* __restrict__ nptr, int* __restrict__ nbr) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= C) return;
  int k = nptr[c];
  const int k0 = k;
  for (int m = ptr[c]; m < ptr[c + 1]; ++m)
    if (nn[m] != m) {
      const int v = m2c[nn[m]];
      int j = k++;
      while (j > k0 && nbr[j - 1] > v) { nbr[j] = nbr[j - 1]; --j; }
      nbr[j] = v;
    }
}

__global__ void k_tail_sum(const int* __restrict__ ex, const int* __restrict__ in, int n, int* __restrict__ out) {
  out[0] = ex[n - 1] + in[n - 1];
}

int total_of(DevBuf& b, const int* ex, const int* in, int n, cudaStream_t s) {
  if (n <= 0) return 0;
  int* d = need<int>(b, 1, "count");
  k_tail_sum<<<1, 1, 0, s>>>(ex, in, n, d);
  int h = 0;
  GEN_CHECK(cudaMemcpyAsync(&h, d, sizeof(int), cudaMemcpyDeviceToHost, s), "count");
  GEN_CHECK(cudaStreamSynchronize(s), "count");
  return h;
}

// bucket the n points (x, y) in cells of side h over [x0, x0 + nx h) x ...
Grid make_grid(DevBuf& b, const double* x, const double* y, int n, double x0, double y0, double h, int nx, int ny,
               cudaStream_t s) {
  uint32_t* key = need<uint32_t>(b, n, "bucket keys");
  int* idx = need<int>(b, n, "bucket index");
  int* start = need<int>(b, (size_t)nx * ny, "buckets");
  int* end = need<int>(b, (size_t)nx * ny, "buckets");
  k_bucket_keys<<<nblocks(n, 256), 256, 0, s>>>(x, y, n, x0, y0, h, nx, ny, key);
  k_iota<<<nblocks(n, 256), 256, 0, s>>>(idx, n);
  int bits = 1;
  while ((1ll << bits) < (int64_t)nx * ny) ++bits;
  radix_sort(b, key, idx, n, bits, s);
  GEN_CHECK(cudaMemsetAsync(start, 0, (size_t)nx * ny * 4, s), "buckets");
  GEN_CHECK(cudaMemsetAsync(end, 0, (size_t)nx * ny * 4, s), "buckets");
  k_bucket_ranges<<<nblocks(n, 256), 256, 0, s>>>(key, n, start, end);
  GEN_CHECK(cudaGetLastError(), "buckets");
  return Grid{x0, y0, h, nx, ny, start, end, idx, x, y, n};
}

// the Delaunay stars of nq queries: the ring walk, then the cells it hands over
void stars(DevBuf& b, const Grid& g, const int* query, int nq, int* nbr, int* nnb, int* flags, cudaStream_t s) {
  SlowCells sc;
  sc.list = need<int>(b, nq, "stars");
  sc.count = need<int>(b, 1, "stars");
  sc.vx = need<double>(b, (size_t)nq * kMaxV, "stars");
  sc.vy = need<double>(b, (size_t)nq * kMaxV, "stars");
  sc.lab = need<int>(b, (size_t)nq * kMaxV, "stars");
  sc.n = need<int>(b, nq, "stars");
  GEN_CHECK(cudaMemsetAsync(sc.count, 0, sizeof(int), s), "stars");
  k_star<<<nblocks(nq, kTpb), kTpb, 0, s>>>(g, query, nq, nbr, nnb, flags, sc);
  int n_slow = 0;
  GEN_CHECK(cudaMemcpyAsync(&n_slow, sc.count, sizeof(int), cudaMemcpyDeviceToHost, s), "stars");
  GEN_CHECK(cudaStreamSynchronize(s), "stars");
  if (n_slow > 0) k_star_scan<<<n_slow, kScanThreads, 0, s>>>(g.px, g.py, g.n, query, sc, nbr, nnb, flags);
  GEN_CHECK(cudaGetLastError(), "stars");
}

}  // namespace

struct bx_generated {
  DevBuf mem;
  int C = 0, M = 0, gny = 0, gnx = 0, n_cell_nn = 0, n_lattice = 0;
  double box[6] = {0, 0, 0, 0, 0, 0};   // xmin, xmax, ymin, ymax, delta, (unused)
  int32_t *ptr = nullptr, *nn = nullptr, *map = nullptr, *cnn_ptr = nullptr, *cnn = nullptr;
  double *sa = nullptr, *nx = nullptr, *ny = nullptr, *rr = nullptr, *mx = nullptr, *my = nullptr;
  double *vol = nullptr, *csa = nullptr, *divi = nullptr, *cx = nullptr, *cy = nullptr, *msa_env = nullptr;
  double *lat_x = nullptr, *lat_y = nullptr;
};

namespace {

void generate(const bx_gen_spec& sp, cudaStream_t s, bx_generated* G) {
  DevBuf tmp;
  DevBuf& keep = G->mem;
  const int64_t N64 = (int64_t)sp.nbx * sp.nby + (int64_t)sp.nrx * sp.nry;
  if (N64 < 4 || N64 > (1ll << 26))
    throw GenError{BX_EINVAL, "bx_generate_cluster: the lattice needs 4 to 2^26 points"};
  const int N = (int)N64;
  G->n_lattice = N;
  // 1. lattice
  uint32_t* words = need<uint32_t>(tmp, 4 * (size_t)N, "random words");
  k_mt19937<<<1, 640, 0, s>>>(sp.seed, 4 * N64, words);
  double* X1 = need<double>(tmp, N + 4, "points");
  double* Y1 = need<double>(tmp, N + 4, "points");
  k_lattice<<<nblocks(N, 256), 256, 0, s>>>(sp, words, X1, Y1);
  double* bnd = need<double>(tmp, 6, "bounds");
  k_bounds<<<1, 1024, 0, s>>>(X1, Y1, N, bnd);
  double hb[6];
  GEN_CHECK(cudaMemcpyAsync(hb, bnd, sizeof(hb), cudaMemcpyDeviceToHost, s), "lattice");
  GEN_CHECK(cudaStreamSynchronize(s), "lattice");
  G->lat_x = need<double>(keep, N, "lattice");
  G->lat_y = need<double>(keep, N, "lattice");
  GEN_CHECK(cudaMemcpyAsync(G->lat_x, X1, (size_t)N * 8, cudaMemcpyDeviceToDevice, s), "lattice");
  GEN_CHECK(cudaMemcpyAsync(G->lat_y, Y1, (size_t)N * 8, cudaMemcpyDeviceToDevice, s), "lattice");
  const double lox = hb[0], hix = hb[1], loy = hb[2], hiy = hb[3];
  const double cenx = hb[4] / N, ceny = hb[5] / N;
  // the bounding-box corners close the first pass's hull (Cells.clust_xy)
  const double corners_x[4] = {lox, hix, hix, lox}, corners_y[4] = {loy, loy, hiy, hiy};
  GEN_CHECK(cudaMemcpyAsync(X1 + N, corners_x, sizeof(corners_x), cudaMemcpyHostToDevice, s), "corners");
  GEN_CHECK(cudaMemcpyAsync(Y1 + N, corners_y, sizeof(corners_y), cudaMemcpyHostToDevice, s), "corners");
  const int N1 = N + 4;

  // 2. pass one, on the lattice points that can have a centroid in the disc
  const double h = sp.d_cell;
  const int gx1 = (int)((hix - lox) / h) + 1, gy1 = (int)((hiy - loy) / h) + 1;
  if ((int64_t)gx1 * gy1 > (1ll << 28)) throw GenError{BX_EINVAL, "bx_generate_cluster: lattice too large"};
  Grid g1 = make_grid(tmp, X1, Y1, N1, lox, loy, h, gx1, gy1, s);
  int* near = need<int>(tmp, N, "query");
  int* near_pos = need<int>(tmp, N, "query");
  k_near_disc<<<nblocks(N, 256), 256, 0, s>>>(X1, Y1, N, cenx, ceny, sp.radius + 3.0 * sp.d_cell, near);
  scan_excl(tmp, near, near_pos, N, s);
  const int nq1 = total_of(tmp, near_pos, near, N, s);
  if (nq1 < 3) throw GenError{BX_EINVAL, "bx_generate_cluster: the disc holds fewer than 3 lattice points"};
  int* q1 = need<int>(tmp, nq1, "query");
  k_compact<<<nblocks(N, 256), 256, 0, s>>>(near, near_pos, N, nullptr, q1);
  int* flags = need<int>(tmp, kNFlags, "flags");
  GEN_CHECK(cudaMemsetAsync(flags, 0, kNFlags * sizeof(int), s), "flags");
  int* nbr1 = need<int>(tmp, (size_t)nq1 * kMaxV, "stars");
  int* nnb1 = need<int>(tmp, nq1, "stars");
  stars(tmp, g1, q1, nq1, nbr1, nnb1, flags, s);
  double* c0x = need<double>(tmp, nq1, "centroids");
  double* c0y = need<double>(tmp, nq1, "centroids");
  int* k1 = need<int>(tmp, nq1, "centroids");
  int* k1p = need<int>(tmp, nq1, "centroids");
  k_pass1<<<nblocks(nq1, kTpb), kTpb, 0, s>>>(X1, Y1, q1, nq1, nbr1, nnb1, cenx, ceny, sp.radius, c0x, c0y, k1, flags);
  GEN_CHECK(cudaGetLastError(), "pass one");
  scan_excl(tmp, k1, k1p, nq1, s);
  const int N2 = total_of(tmp, k1p, k1, nq1, s);
  if (N2 < 4) throw GenError{BX_EINVAL, "bx_generate_cluster: fewer than 4 cell centres in the disc"};
  int* sel = need<int>(tmp, N2, "points");
  k_compact<<<nblocks(nq1, 256), 256, 0, s>>>(k1, k1p, nq1, nullptr, sel);
  double* X2 = need<double>(tmp, N2, "points");
  double* Y2 = need<double>(tmp, N2, "points");
  k_gather2<<<nblocks(N2, 256), 256, 0, s>>>(sel, N2, c0x, c0y, X2, Y2);

  // 3. pass two on the centroids (all within radius of the centre)
  const double x20 = cenx - sp.radius - h, y20 = ceny - sp.radius - h;
  const int gx2 = (int)((2.0 * (sp.radius + h)) / h) + 2, gy2 = gx2;
  Grid g2 = make_grid(tmp, X2, Y2, N2, x20, y20, h, gx2, gy2, s);
  int* nbr2 = need<int>(tmp, (size_t)N2 * kMaxV, "stars");
  int* nnb2 = need<int>(tmp, N2, "stars");
  stars(tmp, g2, nullptr, N2, nbr2, nnb2, flags, s);
  double* PX = need<double>(tmp, (size_t)N2 * kMaxV, "polygons");
  double* PY = need<double>(tmp, (size_t)N2 * kMaxV, "polygons");
  int* other = need<int>(tmp, (size_t)N2 * kMaxV, "polygons");
  int* nv = need<int>(tmp, N2, "polygons");
  double* pcx = need<double>(tmp, N2, "centres");
  double* pcy = need<double>(tmp, N2, "centres");
  int* k2 = need<int>(tmp, N2, "cells");
  int* k2p = need<int>(tmp, N2, "cells");
  k_pass2<<<nblocks(N2, kTpb), kTpb, 0, s>>>(X2, Y2, N2, nbr2, nnb2, PX, PY, other, nv, pcx, pcy, k2, flags);
  GEN_CHECK(cudaGetLastError(), "pass two");
  scan_excl(tmp, k2, k2p, N2, s);
  const int C = total_of(tmp, k2p, k2, N2, s);
  if (C < 1) throw GenError{BX_EINVAL, "bx_generate_cluster: no closed cell"};
  int* seeds = need<int>(tmp, C, "cells");
  k_compact<<<nblocks(N2, 256), 256, 0, s>>>(k2, k2p, N2, nullptr, seeds);

  // 4. cells along the Z curve of their centres
  double* sx = need<double>(tmp, C, "centres");
  double* sy = need<double>(tmp, C, "centres");
  k_gather_centres<<<nblocks(C, 256), 256, 0, s>>>(seeds, C, pcx, pcy, sx, sy);
  double* bnd2 = need<double>(tmp, 6, "bounds");
  k_bounds<<<1, 1024, 0, s>>>(sx, sy, C, bnd2);
  uint32_t* zk = need<uint32_t>(tmp, C, "z keys");
  k_zkeys<<<nblocks(C, 256), 256, 0, s>>>(seeds, C, pcx, pcy, bnd2, zk);
  radix_sort(tmp, zk, seeds, C, 32, s);        // seeds[c]: the point of cell c
  int* counts = need<int>(tmp, C, "cells");
  int* seed_to_cell = need<int>(tmp, N2, "cells");
  GEN_CHECK(cudaMemsetAsync(seed_to_cell, 0xff, (size_t)N2 * 4, s), "cells");
  k_cell_counts<<<nblocks(C, 256), 256, 0, s>>>(seeds, C, nv, counts, seed_to_cell);
  G->ptr = need<int>(keep, C + 1, "cell_mem_ptr");
  scan_excl(tmp, counts, G->ptr, C, s);
  const int M = total_of(tmp, G->ptr, counts, C, s);
  GEN_CHECK(cudaMemcpyAsync(G->ptr + C, &M, sizeof(int), cudaMemcpyHostToDevice, s), "cells");
  G->C = C;
  G->M = M;
  G->mx = need<double>(keep, M, "membranes"); G->my = need<double>(keep, M, "membranes");
  G->nx = need<double>(keep, M, "membranes"); G->ny = need<double>(keep, M, "membranes");
  G->sa = need<double>(keep, M, "membranes"); G->rr = need<double>(keep, M, "membranes");
  G->nn = need<int>(keep, M, "membranes"); G->map = need<int>(keep, M, "membranes");
  int* oth = need<int>(tmp, M, "membranes");
  int* m2c = need<int>(tmp, M, "membranes");
  G->vol = need<double>(keep, C, "cells"); G->csa = need<double>(keep, C, "cells");
  G->divi = need<double>(keep, C, "cells"); G->cx = need<double>(keep, C, "cells");
  G->cy = need<double>(keep, C, "cells");
  k_gather_centres<<<nblocks(C, 256), 256, 0, s>>>(seeds, C, pcx, pcy, G->cx, G->cy);
  k_membranes<<<nblocks(C, kTpb), kTpb, 0, s>>>(seeds, C, G->ptr, PX, PY, other, pcx, pcy, sp.scale_cell,
                                                 sp.cell_height, G->mx, G->my, G->nx, G->ny, G->sa, G->rr, oth, m2c,
                                                 G->vol, G->csa, G->divi);
  k_pair<<<nblocks(M, 256), 256, 0, s>>>(M, m2c, oth, seeds, seed_to_cell, G->ptr, G->nn, flags);
  GEN_CHECK(cudaGetLastError(), "membranes");

  // 5. environment grid (makeECM: the lattice box widened by a cell radius)
  const double xmin = lox - sp.cell_radius, ymin = loy - sp.cell_radius;
  const double xmax = hix + sp.cell_radius, ymax = hiy + sp.cell_radius;
  const double delta = (xmax - xmin) / sp.grid_size;
  const int gnx = (int)((xmax - xmin) / delta), gny = (int)((ymax - ymin) / delta);
  if (gnx < 2 || gny < 2) throw GenError{BX_EINVAL, "bx_generate_cluster: grid_size gives fewer than 2 grid cells"};
  G->gnx = gnx; G->gny = gny;
  G->box[0] = xmin; G->box[1] = xmax; G->box[2] = ymin; G->box[3] = ymax; G->box[4] = delta;
  double* gcx = need<double>(tmp, gnx, "grid");
  double* gcy = need<double>(tmp, gny, "grid");
  k_grid_centres<<<nblocks(gnx, 256), 256, 0, s>>>(xmin, xmax, gnx, gcx);
  k_grid_centres<<<nblocks(gny, 256), 256, 0, s>>>(ymin, ymax, gny, gcy);
  uint32_t* gk = need<uint32_t>(tmp, M, "grid");
  int* gm = need<int>(tmp, M, "grid");
  k_grid_map<<<nblocks(M, 256), 256, 0, s>>>(M, G->mx, G->my, gcx, gnx, gcy, gny, G->map, gk, gm);
  int gbits = 1;
  while ((1ll << gbits) < (int64_t)gnx * gny) ++gbits;
  radix_sort(tmp, gk, gm, M, gbits, s);
  G->msa_env = need<double>(keep, (size_t)gnx * gny, "grid");
  GEN_CHECK(cudaMemsetAsync(G->msa_env, 0, (size_t)gnx * gny * 8, s), "grid");
  k_grid_area<<<nblocks(M, 256), 256, 0, s>>>(M, gk, gm, G->sa, G->msa_env);

  // 6. cell adjacency (near_neigh's cell_nn)
  int* ncnt = need<int>(tmp, C, "adjacency");
  G->cnn_ptr = need<int>(keep, C + 1, "adjacency");
  k_nn_counts<<<nblocks(C, 256), 256, 0, s>>>(C, G->ptr, G->nn, ncnt);
  scan_excl(tmp, ncnt, G->cnn_ptr, C, s);
  const int E = total_of(tmp, G->cnn_ptr, ncnt, C, s);
  GEN_CHECK(cudaMemcpyAsync(G->cnn_ptr + C, &E, sizeof(int), cudaMemcpyHostToDevice, s), "adjacency");
  G->cnn = need<int>(keep, E, "adjacency");
  k_nn_fill<<<nblocks(C, 256), 256, 0, s>>>(C, G->ptr, G->nn, m2c, G->cnn_ptr, G->cnn);
  G->n_cell_nn = E;
  GEN_CHECK(cudaGetLastError(), "adjacency");

  int hf[kNFlags];
  GEN_CHECK(cudaMemcpyAsync(hf, flags, sizeof(hf), cudaMemcpyDeviceToHost, s), "status");
  GEN_CHECK(cudaStreamSynchronize(s), "generation");
  if (hf[kPolyOverflow]) throw GenError{BX_EINVAL, "bx_generate_cluster: a Voronoi cell exceeded 32 vertices"};
  if (hf[kDuplicate]) throw GenError{BX_EINVAL, "bx_generate_cluster: coincident seed points"};
  if (hf[kFanOrder]) throw GenError{BX_EINVAL, "bx_generate_cluster: a triangle fan is not star-shaped"};
  if (hf[kUnpaired])
    throw GenError{BX_EINVAL, "bx_generate_cluster: a shared Delaunay edge is missing from one of its cells"};
}

}  // namespace

extern "C" int bx_generate_cluster(const bx_gen_spec* spec, void* stream, bx_gen_handle* out) {
  if (!spec || !out) {
    bx_record_error("bx_generate_cluster: null argument");
    return BX_EINVAL;
  }
  *out = nullptr;
  if (!(spec->radius > 0.0) || !(spec->d_cell > 0.0) || spec->grid_size < 2 || spec->nbx < 1 || spec->nby < 1 ||
      spec->nrx < 0 || spec->nry < 0 || !(spec->scale_cell > 0.0) || !(spec->cell_height > 0.0)) {
    bx_record_error("bx_generate_cluster: bad specification");
    return BX_EINVAL;
  }
  auto* G = new bx_generated();
  try {
    generate(*spec, static_cast<cudaStream_t>(stream), G);
  } catch (const GenError& e) {
    delete G;
    bx_record_error(e.msg.c_str());
    return e.code;
  }
  *out = G;
  return BX_OK;
}

extern "C" int bx_generated_info(bx_gen_handle g, int32_t* sizes, double* box) {
  if (!g) {
    bx_record_error("bx_generated_info: null handle");
    return BX_EINVAL;
  }
  if (sizes) {
    sizes[0] = g->C; sizes[1] = g->M; sizes[2] = g->gny; sizes[3] = g->gnx;
    sizes[4] = g->n_cell_nn; sizes[5] = g->n_lattice;
  }
  if (box)
    for (int k = 0; k < 5; ++k) box[k] = g->box[k];
  return BX_OK;
}

extern "C" int bx_generated_download(bx_gen_handle g, const bx_gen_arrays* a) {
  if (!g || !a) {
    bx_record_error("bx_generated_download: null argument");
    return BX_EINVAL;
  }
  struct Item { void* dst; const void* src; size_t bytes; };
  const size_t C = g->C, M = g->M, G = (size_t)g->gny * g->gnx, E = g->n_cell_nn, L = g->n_lattice;
  const Item items[] = {
      {a->cell_mem_ptr, g->ptr, (C + 1) * 4}, {a->nn_i, g->nn, M * 4}, {a->map_mem2ecm, g->map, M * 4},
      {a->mem_sa, g->sa, M * 8}, {a->mem_nx, g->nx, M * 8}, {a->mem_ny, g->ny, M * 8},
      {a->R_rads, g->rr, M * 8}, {a->mem_mid_x, g->mx, M * 8}, {a->mem_mid_y, g->my, M * 8},
      {a->cell_vol, g->vol, C * 8}, {a->cell_sa, g->csa, C * 8}, {a->diviterm, g->divi, C * 8},
      {a->cell_centre_x, g->cx, C * 8}, {a->cell_centre_y, g->cy, C * 8},
      {a->mem_sa_per_env, g->msa_env, G * 8}, {a->cell_nn_ptr, g->cnn_ptr, (C + 1) * 4},
      {a->cell_nn, g->cnn, E * 4}, {a->lattice_x, g->lat_x, L * 8}, {a->lattice_y, g->lat_y, L * 8}};
  for (const Item& it : items)
    if (it.dst && it.bytes && cudaMemcpy(it.dst, it.src, it.bytes, cudaMemcpyDefault) != cudaSuccess) {
      bx_record_error("bx_generated_download: copy failed");
      return BX_ECUDA;
    }
  return BX_OK;
}

extern "C" int bx_generated_destroy(bx_gen_handle g) {
  delete g;
  return BX_OK;
}
