// Two-way-coupling deposition, FP64 drop-in form. No atomics anywhere: every
// target value is a sum in a fixed order, so results are identical run to run.
//
// Fast path (k_dep_brick): one CTA per brick of B^3 target cells of the ghosted
// grid. Its threads walk the CSR segments (particles sorted by node, then h,
// then storage index) of the brick's nodes plus a one-node halo, form per-node
// partial sums in shared memory -- the 8 trilinear offsets of a node, and the
// face-normal partials of each trunc cell, added in 8 conflict-free phases (one
// per h class) -- then every target cell sums its partials in a fixed order.
// Halo nodes are walked by both neighbouring bricks; no cross-brick reduction.
//
// Reference-order path (PSTEP_REFERENCE_SUMS, k_dep_trilinear / k_dep_face):
// each thread owns one target cell and merges the node lists by the particles'
// positions in the reference's vectors, so every cell receives its
// contributions in exactly the order the reference's scatter loop adds them
// (particle.cpp:498-658), from 0, with the reference's weight expressions.
// Either way the cumulative ghost fold and the ghost refresh then replay
// communicator.cpp's single-rank sequence.
//
// Compiled with -fmad=false (see stage_f64.cu).
#include "pstep_internal.cuh"

namespace pstep {
namespace {

struct DepIn {
  const int32_t *cell_start;  // gsize + 1
  const int32_t *sidx;        // nullptr: identity
  const int32_t *order;       // secondary key per particle (nullptr: storage index)
  const double *frac[3];
  const uint32_t *key;
  const double *val[3];       // RHS_u,v,w (int-deposit) or RHS_T in val[0] (temperature deposit)
};

__device__ inline int32_t pidx(const DepIn &d, int32_t p) { return d.sidx ? d.sidx[p] : p; }
__device__ inline int32_t okey(const DepIn &d, int32_t q) { return d.order ? d.order[q] : q; }

// K-way merge over node segments, calling f(particle) in ascending secondary-key order.
template <int K, typename F>
__device__ inline void merge_walk(const DepIn &d, const long long (&nodes)[K], F f) {
  int32_t cur[K], end[K], head[K];
#pragma unroll
  for (int q = 0; q < K; ++q) {
    if (nodes[q] >= 0) {
      cur[q] = d.cell_start[nodes[q]];
      end[q] = d.cell_start[nodes[q] + 1];
    } else {
      cur[q] = 0;
      end[q] = 0;
    }
    head[q] = cur[q] < end[q] ? okey(d, pidx(d, cur[q])) : INT32_MAX;
  }
  while (true) {
    int best = -1;
    int32_t bk = INT32_MAX;
#pragma unroll
    for (int q = 0; q < K; ++q)
      if (head[q] < bk) { bk = head[q]; best = q; }
    if (best < 0) break;
#pragma unroll
    for (int q = 0; q < K; ++q)
      if (q == best) {
        f(pidx(d, cur[q]), q);
        ++cur[q];
        head[q] = cur[q] < end[q] ? okey(d, pidx(d, cur[q])) : INT32_MAX;
      }
  }
}

__device__ inline bool node_ok(const Geom &G, int i, int j, int k) {
  // particle nodes are round(x*idx)+1 in 1..n+1
  return i >= 1 && i <= G.n[0] + 1 && j >= 1 && j <= G.n[1] + 1 && k >= 1 && k <= G.n[2] + 1;
}

__device__ inline double xl_round(double f, int h) { return (h ? (f - 1.0) : f) + 0.5; }

// Trilinear deposit (concentration weights, or weights * RHS_T) into target t:
// contributions come from nodes t + {0,1}^3; offset o = node - t selects the
// factor (o ? 1 - x_l : x_l) per dimension, combined as ((fx*fy)*fz)[*val] --
// the operand order of every term in particle.cpp:548-555 and :645-652.
__global__ void k_dep_trilinear(Geom G, DepIn d, int with_val, double *__restrict__ out) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= G.gsize) return;
  const int ti = (int)(t % G.g[0]);
  const int tj = (int)((t / G.g[0]) % G.g[1]);
  const int tk = (int)(t / ((long long)G.g[0] * G.g[1]));
  long long nodes[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    int ox = (q >> 2) & 1, oy = (q >> 1) & 1, oz = q & 1;
    int ni = ti + ox, nj = tj + oy, nk = tk + oz;
    nodes[q] = node_ok(G, ni, nj, nk) ? glin(G, ni, nj, nk) : -1;
  }
  double acc = 0.0;
  merge_walk<8>(d, nodes, [&](int32_t p, int q) {
    const uint32_t key = d.key[p];
    const int ox = (q >> 2) & 1, oy = (q >> 1) & 1, oz = q & 1;
    const double xl = xl_round(d.frac[0][p], (key >> 2) & 1);
    const double yl = xl_round(d.frac[1][p], (key >> 1) & 1);
    const double zl = xl_round(d.frac[2][p], key & 1);
    const double fx = ox ? (1 - xl) : xl;
    const double fy = oy ? (1 - yl) : yl;
    const double fz = oz ? (1 - zl) : zl;
    double w = fx * fy * fz;
    if (with_val) w = w * d.val[0][p];
    acc += w;
  });
  out[t] = acc;
}

// Face-normal momentum deposit (particle.cpp:498-524): x-face t receives
// x_l*RHS_u from particles whose trunc cell (ghosted) is (ti-1, tj, tk) and
// (1-x_l)*RHS_u from those in (ti, tj, tk); trunc cell = node - h.
template <int D>
__global__ void k_dep_face(Geom G, DepIn d, double *__restrict__ out) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= G.gsize) return;
  const int tc[3] = {(int)(t % G.g[0]), (int)((t / G.g[0]) % G.g[1]), (int)(t / ((long long)G.g[0] * G.g[1]))};
  // nodes: along D in {t-1, t, t+1}, across in {t, t+1}
  long long nodes[12];
#pragma unroll
  for (int q = 0; q < 12; ++q) {
    int a = q / 4 - 1, b = (q >> 1) & 1, c = q & 1;
    int n3[3];
    n3[D] = tc[D] + a;
    n3[(D + 1) % 3] = tc[(D + 1) % 3] + b;
    n3[(D + 2) % 3] = tc[(D + 2) % 3] + c;
    nodes[q] = node_ok(G, n3[0], n3[1], n3[2]) ? glin(G, n3[0], n3[1], n3[2]) : -1;
  }
  double acc = 0.0;
  merge_walk<12>(d, nodes, [&](int32_t p, int q) {
    const uint32_t key = d.key[p];
    const long long lin = key >> 3;
    const int h3[3] = {(int)((key >> 2) & 1), (int)((key >> 1) & 1), (int)(key & 1)};
    const int n3[3] = {(int)(lin % G.g[0]), (int)((lin / G.g[0]) % G.g[1]),
                       (int)(lin / ((long long)G.g[0] * G.g[1]))};
    const int c0 = n3[D] - h3[D];
    const int c1 = n3[(D + 1) % 3] - h3[(D + 1) % 3];
    const int c2 = n3[(D + 2) % 3] - h3[(D + 2) % 3];
    if (c1 != tc[(D + 1) % 3] || c2 != tc[(D + 2) % 3]) return;
    const double xl = d.frac[D][p];
    if (c0 == tc[D] - 1) acc += xl * d.val[D][p];
    else if (c0 == tc[D]) acc += (1 - xl) * d.val[D][p];
  });
  out[t] = acc;
}

// ---- fast path ----------------------------------------------------------------
constexpr int kB = 8;                 // brick edge (target cells)
constexpr int kB1 = kB + 1;           // trilinear node region edge [b, b+B]
constexpr int kB2 = kB + 2;           // face node region edge [b-1, b+B]
constexpr int kBrickThreads = 256;
constexpr size_t kBrickSmem = (size_t)kB1 * kB1 * kB1 * (8 + 6) * sizeof(double);
// A node (or node h-class segment) with more particles than this is summed by a
// warp: lanes stride its particles in order and a fixed shuffle tree adds the
// lane sums. The order is fixed by the segment alone, so the result is the same
// from run to run; one thread walking a blob-centre node (~1000 particles)
// would hold up its whole brick.
constexpr int kDenseSeg = 32;
constexpr int kDenseMax = kB2 * kB2 * kB2;

__device__ __forceinline__ double warp_tree_sum(double v) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
  return v;  // lane 0 holds the sum
}

// The fast deposit sums moments per node instead of the 8 corner weights: with
// t = (x_l, y_l, z_l) of each particle and value v (1 for the concentration),
// M[s] = sum v * prod_{d in s} t_d for the 8 subsets s of {x (4), y (2), z (1)}.
// The corner with (1 - t_d) in the dimensions of bit set o and t_d in the others is
// sum_{A subset of o} (-1)^|A| M[A | ~o], formed once per node. GB300's FP64 pipe
// is the bound of this kernel, and per particle this takes 3 + 4 + 8 FP64
// operations instead of 6 + 3 + 24 (+ 8). x_l = frac + 0.5 - h is formed as
// frac + (h ? -0.5 : 0.5), the same value (frac - 1 and frac - 0.5 are exact for
// frac >= 0.5).
__device__ __forceinline__ void moments_add(double (&m)[8], const DepIn &d, int32_t p, int mode) {
  const uint32_t key = d.key[p];
  const double xl = d.frac[0][p] + (((key >> 2) & 1) ? -0.5 : 0.5);
  const double yl = d.frac[1][p] + (((key >> 1) & 1) ? -0.5 : 0.5);
  const double zl = d.frac[2][p] + ((key & 1) ? -0.5 : 0.5);
  const double xy = xl * yl, xz = xl * zl, yz = yl * zl, xyz = xy * zl;
  if (mode) {
    const double v = d.val[0][p];
    m[0] += v;
    m[4] = fma(xl, v, m[4]);
    m[2] = fma(yl, v, m[2]);
    m[1] = fma(zl, v, m[1]);
    m[6] = fma(xy, v, m[6]);
    m[5] = fma(xz, v, m[5]);
    m[3] = fma(yz, v, m[3]);
    m[7] = fma(xyz, v, m[7]);
  } else {
    m[0] += 1.0;
    m[4] += xl;
    m[2] += yl;
    m[1] += zl;
    m[6] += xy;
    m[5] += xz;
    m[3] += yz;
    m[7] += xyz;
  }
}

// corner partial o (bit 2: x takes 1 - x_l, bit 1: y, bit 0: z) from the moments
__device__ __forceinline__ double corner_of(const double (&m)[8], int o) {
  const int rest = ~o & 7;
  double c = 0.0;
#pragma unroll
  for (int a = 0; a < 8; ++a) {
    if ((a & o) != a) continue;  // subsets of o only
    const double t = m[a | rest];
    c = (__popc(a) & 1) ? c - t : c + t;
  }
  return c;
}

// face sums of one particle: (sum r, sum t r) per dimension, r = RHS_u component
__device__ __forceinline__ void face_add(double (&f)[6], const DepIn &d, int32_t p) {
#pragma unroll
  for (int D = 0; D < 3; ++D) {
    const double r = d.val[D][p];
    f[2 * D] += r;
    f[2 * D + 1] = fma(d.frac[D][p], r, f[2 * D + 1]);
  }
}

__device__ inline int32_t seg_lower_h(const DepIn &d, int32_t a, int32_t b, uint32_t hcls) {
  // first position in [a, b) whose particle has h class >= hcls (segments are sorted by h)
  while (a < b) {
    int32_t m = (a + b) >> 1;
    if ((d.key[pidx(d, m)] & 7u) < hcls) a = m + 1; else b = m;
  }
  return a;
}

// mode 0: concentration (weights) + face momentum partials at x_int; mode 1: weights * RHS_T
//
// A pre-pass tabulates, for every node of the brick's region [b-1, b+B], where its
// segment starts and where each h class ends inside it (segments are sorted by h):
// short segments by reading their keys (independent loads), longer ones by binary
// search, each once per brick rather than once per phase. Nodes whose segment is
// too long for 16-bit class ends (none at the particle densities of the workloads)
// fall back to the searches in every phase.
__global__ void __launch_bounds__(kBrickThreads) k_dep_brick(Geom G, DepIn d, int mode, int twc,
                                                             double *__restrict__ out_tri,
                                                             double *__restrict__ out_x,
                                                             double *__restrict__ out_y,
                                                             double *__restrict__ out_z) {
  extern __shared__ double sm[];
  double *P = sm;                              // [kB1^3][8] trilinear partials of node b + l
  double *F = sm + kB1 * kB1 * kB1 * 8;        // [kB1^3][6] face partials of trunc cell b - 1 + l
  __shared__ int32_t seg_a[kDenseMax];         // node b - 1 + l: first sorted position
  __shared__ uint16_t cls_end[kDenseMax][8];   // end of h classes 0..hc, relative to seg_a
  __shared__ int32_t dense_s[kDenseMax];
  __shared__ int32_t n_dense;
  constexpr uint16_t kUntabulated = 0xffffu;
  const int nbx = (G.g[0] + kB - 1) / kB, nby = (G.g[1] + kB - 1) / kB;
  const int bx = (int)(blockIdx.x % nbx) * kB;
  const int by = (int)((blockIdx.x / nbx) % nby) * kB;
  const int bz = (int)(blockIdx.x / ((long long)nbx * nby)) * kB;
  const int lane = (int)(threadIdx.x & 31u), warp = (int)(threadIdx.x >> 5), nwarps = kBrickThreads / 32;

  // pre-pass: segment table of the region's nodes
  for (int s = threadIdx.x; s < kB2 * kB2 * kB2; s += blockDim.x) {
    const int lx = s % kB2, ly = (s / kB2) % kB2, lz = s / (kB2 * kB2);
    const int ni = bx - 1 + lx, nj = by - 1 + ly, nk = bz - 1 + lz;
    int32_t a0 = 0, cnt = 0;
    if (node_ok(G, ni, nj, nk)) {
      const long long n = glin(G, ni, nj, nk);
      a0 = d.cell_start[n];
      cnt = d.cell_start[n + 1] - a0;
    }
    seg_a[s] = a0;
    if (cnt <= 16) {
      uint64_t c = 0;  // 8 one-byte class counts (at most 16 each)
      for (int32_t q = 0; q < cnt; ++q) c += 1ull << (8u * (d.key[pidx(d, a0 + q)] & 7u));
      int run = 0;
#pragma unroll
      for (int hc = 0; hc < 8; ++hc) {
        run += (int)((c >> (8 * hc)) & 0xffu);
        cls_end[s][hc] = (uint16_t)run;
      }
    } else if (cnt < (int32_t)kUntabulated) {
#pragma unroll 1
      for (int hc = 0; hc < 7; ++hc) cls_end[s][hc] = (uint16_t)(seg_lower_h(d, a0, a0 + cnt, hc + 1) - a0);
      cls_end[s][7] = (uint16_t)cnt;
    } else {
      cls_end[s][7] = kUntabulated;
    }
  }
  if (threadIdx.x == 0) n_dense = 0;
  __syncthreads();
  // [a, e) of node slot s (region index) and h class hc
  auto seg = [&](int s, int hc, int32_t &a, int32_t &e) {
    const int32_t a0 = seg_a[s];
    if (cls_end[s][7] != kUntabulated) {
      a = a0 + (hc ? cls_end[s][hc - 1] : 0);
      e = a0 + cls_end[s][hc];
    } else {  // a segment longer than the table holds
      const int lx = s % kB2, ly = (s / kB2) % kB2, lz = s / (kB2 * kB2);
      const long long n = glin(G, bx - 1 + lx, by - 1 + ly, bz - 1 + lz);
      const int32_t e0 = d.cell_start[n + 1];
      a = hc ? seg_lower_h(d, a0, e0, hc) : a0;
      e = hc < 7 ? seg_lower_h(d, a, e0, hc + 1) : e0;
    }
  };
  // whole segment of node slot s
  auto whole = [&](int s, int32_t &a, int32_t &e) {
    int32_t a1, e1;
    seg(s, 0, a, e1);
    seg(s, 7, a1, e);
  };

  // trilinear: per-node partials for nodes [b, b+B] (region slot = l + 1); dense nodes listed for the warps
  for (int s = threadIdx.x; s < kB1 * kB1 * kB1; s += blockDim.x) {
    const int lx = s % kB1, ly = (s / kB1) % kB1, lz = s / (kB1 * kB1);
    const int rs = ((lz + 1) * kB2 + (ly + 1)) * kB2 + (lx + 1);
    double m[8];
#pragma unroll
    for (int o = 0; o < 8; ++o) m[o] = 0.0;
    int32_t a, e;
    whole(rs, a, e);
    if (e - a > kDenseSeg) {
      dense_s[atomicAdd(&n_dense, 1)] = s;
      continue;
    }
    // one path for every node (empty ones included): the FP64 pipe is charged per warp
    // instruction, so lanes on different paths would cost the warp both
    for (int32_t q = a; q < e; ++q) moments_add(m, d, pidx(d, q), mode);
#pragma unroll
    for (int o = 0; o < 8; ++o) P[s * 8 + o] = corner_of(m, o);
  }
  __syncthreads();
  for (int k = warp; k < n_dense; k += nwarps) {
    const int s = dense_s[k];
    const int lx = s % kB1, ly = (s / kB1) % kB1, lz = s / (kB1 * kB1);
    int32_t a, e;
    whole(((lz + 1) * kB2 + (ly + 1)) * kB2 + (lx + 1), a, e);
    double m[8];
#pragma unroll
    for (int o = 0; o < 8; ++o) m[o] = 0.0;
    for (int32_t q = a + lane; q < e; q += 32) moments_add(m, d, pidx(d, q), mode);
#pragma unroll
    for (int o = 0; o < 8; ++o) m[o] = warp_tree_sum(m[o]);
    if (lane == 0) {
#pragma unroll
      for (int o = 0; o < 8; ++o) P[s * 8 + o] = corner_of(m, o);
    }
  }
  const bool faces = (mode == 0) && twc;
  if (faces) {
    for (int s = threadIdx.x; s < kB1 * kB1 * kB1 * 6; s += blockDim.x) F[s] = 0.0;
  }
  __syncthreads();
  // face partials: trunc cell c = node - h, one h class per phase (distinct nodes -> distinct cells);
  // dense segments listed for the warps as above
  if (faces) {
    for (int hc = 0; hc < 8; ++hc) {
      const int hx = (hc >> 2) & 1, hy = (hc >> 1) & 1, hz = hc & 1;
      if (threadIdx.x == 0) n_dense = 0;
      __syncthreads();
      for (int s = threadIdx.x; s < kB2 * kB2 * kB2; s += blockDim.x) {
        const int lx = s % kB2, ly = (s / kB2) % kB2, lz = s / (kB2 * kB2);
        const int cx = lx - hx, cy = ly - hy, cz = lz - hz;  // cell slot: cell = b - 1 + c
        if (cx < 0 || cy < 0 || cz < 0 || cx >= kB1 || cy >= kB1 || cz >= kB1) continue;
        int32_t a, e;
        seg(s, hc, a, e);
        if (a == e) continue;
        if (e - a > kDenseSeg) {
          dense_s[atomicAdd(&n_dense, 1)] = s;
          continue;
        }
        double fs[6] = {0, 0, 0, 0, 0, 0};
        for (int32_t q = a; q < e; ++q) face_add(fs, d, pidx(d, q));
        // (1 - x_l) r summed as sum r - sum x_l r; x_l r as is
        double *f = F + ((cz * kB1 + cy) * kB1 + cx) * 6;
#pragma unroll
        for (int D = 0; D < 3; ++D) {
          f[2 * D] += fs[2 * D] - fs[2 * D + 1];
          f[2 * D + 1] += fs[2 * D + 1];
        }
      }
      __syncthreads();
      for (int k = warp; k < n_dense; k += nwarps) {
        const int s = dense_s[k];
        const int lx = s % kB2, ly = (s / kB2) % kB2, lz = s / (kB2 * kB2);
        const int cx = lx - hx, cy = ly - hy, cz = lz - hz;
        int32_t a, e;
        seg(s, hc, a, e);
        double fs[6] = {0, 0, 0, 0, 0, 0};
        for (int32_t q = a + lane; q < e; q += 32) face_add(fs, d, pidx(d, q));
#pragma unroll
        for (int j = 0; j < 6; ++j) fs[j] = warp_tree_sum(fs[j]);
        if (lane == 0) {
          double *f = F + ((cz * kB1 + cy) * kB1 + cx) * 6;
#pragma unroll
          for (int D = 0; D < 3; ++D) {
            f[2 * D] += fs[2 * D] - fs[2 * D + 1];
            f[2 * D + 1] += fs[2 * D + 1];
          }
        }
      }
      __syncthreads();
    }
  }
  // targets of the brick
  for (int s = threadIdx.x; s < kB * kB * kB; s += blockDim.x) {
    const int lx = s % kB, ly = (s / kB) % kB, lz = s / (kB * kB);
    const int ti = bx + lx, tj = by + ly, tk = bz + lz;
    if (ti >= G.g[0] || tj >= G.g[1] || tk >= G.g[2]) continue;
    double acc = 0.0;
#pragma unroll
    for (int o = 0; o < 8; ++o) {
      const int ox = (o >> 2) & 1, oy = (o >> 1) & 1, oz = o & 1;
      acc += P[(((lz + oz) * kB1 + (ly + oy)) * kB1 + (lx + ox)) * 8 + o];
    }
    const long long t = glin(G, ti, tj, tk);
    out_tri[t] = acc;
    if (faces) {
      // cell slot of target cell t is l + 1; its lower neighbour in dimension D is l
      const double *ft = F + (((lz + 1) * kB1 + (ly + 1)) * kB1 + (lx + 1)) * 6;
      const double *fxm = F + (((lz + 1) * kB1 + (ly + 1)) * kB1 + lx) * 6;
      const double *fym = F + (((lz + 1) * kB1 + ly) * kB1 + (lx + 1)) * 6;
      const double *fzm = F + ((lz * kB1 + (ly + 1)) * kB1 + (lx + 1)) * 6;
      out_x[t] = fxm[1] + ft[0];
      out_y[t] = fym[3] + ft[2];
      out_z[t] = fzm[5] + ft[4];
    }
  }
}

// communicator.cpp:422-511 on one rank, one phase per launch; nf fields at once
struct FieldSet {
  double *f[5];
  int nf;
};

__global__ void k_fold_z(Geom G, FieldSet fs) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long plane = (long long)G.g[0] * G.g[1];
  if (t >= plane * fs.nf) return;
  int q = (int)(t / plane);
  long long ij = t % plane;
  double *f = fs.f[q];
  const int K = G.g[2];
  double top = f[(long long)(K - 1) * plane + ij], bot = f[ij];
  f[(long long)(K - 2) * plane + ij] += bot;
  f[plane + ij] += top;
}

__global__ void k_fold_y(Geom G, FieldSet fs) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long per = (long long)G.g[0] * G.n[2];
  if (t >= per * fs.nf) return;
  int q = (int)(t / per);
  long long r = t % per;
  int i = (int)(r % G.g[0]), k = (int)(r / G.g[0]) + 1;
  double *f = fs.f[q];
  const int J = G.g[1];
  double top = f[glin(G, i, J - 1, k)], bot = f[glin(G, i, 0, k)];
  f[glin(G, i, J - 2, k)] += bot;
  f[glin(G, i, 1, k)] += top;
}

__global__ void k_fold_x(Geom G, FieldSet fs) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long per = (long long)G.n[1] * G.n[2];
  if (t >= per * fs.nf) return;
  int q = (int)(t / per);
  long long r = t % per;
  int j = (int)(r % G.n[1]) + 1, k = (int)(r / G.n[1]) + 1;
  double *f = fs.f[q];
  const int I = G.g[0];
  double top = f[glin(G, I - 1, j, k)], bot = f[glin(G, 0, j, k)];
  f[glin(G, I - 2, j, k)] += bot;
  f[glin(G, 1, j, k)] += top;
}

// communicator.cpp:177-278 on one rank: x (interior j,k), y (all i, interior k), z (all i,j)
__global__ void k_refresh_x(Geom G, FieldSet fs) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long per = (long long)G.n[1] * G.n[2];
  if (t >= per * fs.nf) return;
  int q = (int)(t / per);
  long long r = t % per;
  int j = (int)(r % G.n[1]) + 1, k = (int)(r / G.n[1]) + 1;
  double *f = fs.f[q];
  const int I = G.g[0];
  f[glin(G, I - 1, j, k)] = f[glin(G, 1, j, k)];
  f[glin(G, 0, j, k)] = f[glin(G, I - 2, j, k)];
}

__global__ void k_refresh_y(Geom G, FieldSet fs) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long per = (long long)G.g[0] * G.n[2];
  if (t >= per * fs.nf) return;
  int q = (int)(t / per);
  long long r = t % per;
  int i = (int)(r % G.g[0]), k = (int)(r / G.g[0]) + 1;
  double *f = fs.f[q];
  const int J = G.g[1];
  f[glin(G, i, J - 1, k)] = f[glin(G, i, 1, k)];
  f[glin(G, i, 0, k)] = f[glin(G, i, J - 2, k)];
}

__global__ void k_refresh_z(Geom G, FieldSet fs) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long plane = (long long)G.g[0] * G.g[1];
  if (t >= plane * fs.nf) return;
  int q = (int)(t / plane);
  long long ij = t % plane;
  double *f = fs.f[q];
  const int K = G.g[2];
  f[(long long)(K - 1) * plane + ij] = f[plane + ij];
  f[ij] = f[(long long)(K - 2) * plane + ij];
}

// Interior sum, fixed order: per-block tree over a strided range, then one block.
constexpr int kRedBlocks = 1024;
__global__ void k_sum_partial(Geom G, const double *__restrict__ f, double *__restrict__ part) {
  __shared__ double sm[kThreads];
  // rows (j,k) distributed over blocks, the i loop over threads: fixed order, coalesced
  const long long rows = (long long)G.n[1] * G.n[2];
  double s = 0.0;
  for (long long r = blockIdx.x; r < rows; r += gridDim.x) {
    const int j = (int)(r % G.n[1]) + 1, k = (int)(r / G.n[1]) + 1;
    const double *row = f + glin(G, 0, j, k);
    for (int i = threadIdx.x + 1; i <= G.n[0]; i += blockDim.x) s += row[i];
  }
  sm[threadIdx.x] = s;
  __syncthreads();
  for (int o = kThreads / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sm[threadIdx.x] += sm[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sm[0];
}

__global__ void k_sum_final(const double *__restrict__ part, int np, double inv_count, double *__restrict__ out) {
  __shared__ double sm[kThreads];
  double s = 0.0;
  for (int i = threadIdx.x; i < np; i += kThreads) s += part[i];
  sm[threadIdx.x] = s;
  __syncthreads();
  for (int o = kThreads / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sm[threadIdx.x] += sm[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sm[0] * inv_count;
}

inline int blocks_for(long long n) { return (int)((n + kThreads - 1) / kThreads); }

DepIn make_in(pstep_ctx *h, const Csr &csr, double *const frac[3], const uint32_t *key, const double *v0,
              const double *v1, const double *v2) {
  DepIn d;
  d.cell_start = csr.cell_start;
  d.sidx = csr.identity ? nullptr : csr.sidx;
  d.order = ((h->cfg.flags & PSTEP_TRACK_ORDER) && (h->cfg.flags & PSTEP_REFERENCE_SUMS)) ? h->ref_of_phys : nullptr;
  for (int q = 0; q < 3; ++q) d.frac[q] = frac[q];
  d.key = key;
  d.val[0] = v0;
  d.val[1] = v1;
  d.val[2] = v2;
  return d;
}

}  // namespace

// refresh: 0 fold only, 1 fold then refresh, 2 refresh only (interior already periodic)
int fold_fields(pstep_ctx *h, double *const *f, int nf, int refresh) {
  const Geom &G = h->geom;
  FieldSet fs;
  fs.nf = nf;
  for (int q = 0; q < nf; ++q) fs.f[q] = f[q];
  long long plane = (long long)G.g[0] * G.g[1];
  if (refresh == 2) {
    k_refresh_x<<<blocks_for((long long)G.n[1] * G.n[2] * nf), kThreads, 0, h->stream>>>(G, fs);
    PSTEP_LAUNCHED(h);
    k_refresh_y<<<blocks_for((long long)G.g[0] * G.n[2] * nf), kThreads, 0, h->stream>>>(G, fs);
    PSTEP_LAUNCHED(h);
    k_refresh_z<<<blocks_for(plane * nf), kThreads, 0, h->stream>>>(G, fs);
    PSTEP_LAUNCHED(h);
    return PSTEP_OK;
  }
  k_fold_z<<<blocks_for(plane * nf), kThreads, 0, h->stream>>>(G, fs);
  PSTEP_LAUNCHED(h);
  k_fold_y<<<blocks_for((long long)G.g[0] * G.n[2] * nf), kThreads, 0, h->stream>>>(G, fs);
  PSTEP_LAUNCHED(h);
  k_fold_x<<<blocks_for((long long)G.n[1] * G.n[2] * nf), kThreads, 0, h->stream>>>(G, fs);
  PSTEP_LAUNCHED(h);
  if (refresh) {
    k_refresh_x<<<blocks_for((long long)G.n[1] * G.n[2] * nf), kThreads, 0, h->stream>>>(G, fs);
    PSTEP_LAUNCHED(h);
    k_refresh_y<<<blocks_for((long long)G.g[0] * G.n[2] * nf), kThreads, 0, h->stream>>>(G, fs);
    PSTEP_LAUNCHED(h);
    k_refresh_z<<<blocks_for(plane * nf), kThreads, 0, h->stream>>>(G, fs);
    PSTEP_LAUNCHED(h);
  }
  return PSTEP_OK;
}

int interior_mean(pstep_ctx *h, const double *f, double *out_dev) {
  const Geom &G = h->geom;
  k_sum_partial<<<kRedBlocks, kThreads, 0, h->stream>>>(G, f, h->red_partials);
  PSTEP_LAUNCHED(h);
  double inv = 1.0 / (double)((long long)G.n[0] * G.n[1] * G.n[2]);
  k_sum_final<<<1, kThreads, 0, h->stream>>>(h->red_partials, kRedBlocks, inv, out_dev);
  PSTEP_LAUNCHED(h);
  return PSTEP_OK;
}

// The momentum balance of the last int deposit: the interior sums of RHS_RU x/y/z,
// each in the fixed order of k_sum_partial / k_sum_final (zeros without TWC).
int momentum_sums(pstep_ctx *h) {
  const Geom &G = h->geom;
  if (!h->cfg.twc) {
    PSTEP_CUDA(cudaMemsetAsync(h->mom_dev, 0, 3 * sizeof(double), h->stream));
    return PSTEP_OK;
  }
  for (int d = 0; d < 3; ++d) {
    double *part = h->red_partials + (1 + d) * kRedBlocks;
    k_sum_partial<<<kRedBlocks, kThreads, 0, h->stream>>>(G, h->dep[PSTEP_FIELD_RU_X + d], part);
    PSTEP_LAUNCHED(h);
    k_sum_final<<<1, kThreads, 0, h->stream>>>(part, kRedBlocks, 1.0, h->mom_dev + d);
    PSTEP_LAUNCHED(h);
  }
  return PSTEP_OK;
}

// part2gas_Temp_int/new: deposit RHS_T with the records of csr/frac/key, fold, refresh, mean.
bool reference_sums(const pstep_ctx *h) {
  return (h->cfg.flags & PSTEP_TRACK_ORDER) && (h->cfg.flags & PSTEP_REFERENCE_SUMS);
}

int brick_launch(pstep_ctx *h, const DepIn &d, int mode, double *tri, double *ox, double *oy, double *oz) {
  const Geom &G = h->geom;
  // the opt-in applies to the current device, which is the one this launch uses;
  // setting it at every launch keeps it right for handles on several devices
  PSTEP_CUDA(cudaFuncSetAttribute(k_dep_brick, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kBrickSmem));
  const long long nb = (long long)((G.g[0] + kB - 1) / kB) * ((G.g[1] + kB - 1) / kB) * ((G.g[2] + kB - 1) / kB);
  k_dep_brick<<<(unsigned)nb, kBrickThreads, kBrickSmem, h->stream>>>(G, d, mode, h->cfg.twc, tri, ox, oy, oz);
  PSTEP_LAUNCHED(h);
  return PSTEP_OK;
}

int deposit_temperature(pstep_ctx *h, const Csr &csr, double *const frac[3], const uint32_t *key) {
  const Geom &G = h->geom;
  DepIn d = make_in(h, csr, frac, key, h->s.rhs_t, nullptr, nullptr);
  double *out = h->dep[PSTEP_FIELD_PART_TEMP];
  if (reference_sums(h)) {
    k_dep_trilinear<<<blocks_for(G.gsize), kThreads, 0, h->stream>>>(G, d, 1, out);
    PSTEP_LAUNCHED(h);
  } else {
    int rc = brick_launch(h, d, 1, out, nullptr, nullptr, nullptr);
    if (rc) return rc;
  }
  double *fl[1] = {out};
  int rc = fold_fields(h, fl, 1, 1);
  if (rc) return rc;
  return interior_mean(h, out, h->emean_dev);
}

// part2gas_concentration + part2gas_velocity at x_int (records of the previous CSR)
int f64_deposit_int(pstep_ctx *h) {
  const Geom &G = h->geom;
  DepIn d = make_in(h, h->csr_prev, h->s.frac_prev, h->s.key_prev, h->s.rhs_u[0], h->s.rhs_u[1], h->s.rhs_u[2]);
  if (!reference_sums(h)) {
    int rc = brick_launch(h, d, 0, h->dep[PSTEP_FIELD_C], h->dep[PSTEP_FIELD_RU_X], h->dep[PSTEP_FIELD_RU_Y],
                          h->dep[PSTEP_FIELD_RU_Z]);
    if (rc) return rc;
    double *c1[1] = {h->dep[PSTEP_FIELD_C]};
    rc = fold_fields(h, c1, 1, 0);  // the reference does not refresh C's ghosts
    if (rc) return rc;
    if (h->cfg.twc) {
      double *ru[3] = {h->dep[PSTEP_FIELD_RU_X], h->dep[PSTEP_FIELD_RU_Y], h->dep[PSTEP_FIELD_RU_Z]};
      rc = fold_fields(h, ru, 3, 1);
      if (rc) return rc;
    } else {
      for (int q = PSTEP_FIELD_RU_X; q <= PSTEP_FIELD_RU_Z; ++q)
        PSTEP_CUDA(cudaMemsetAsync(h->dep[q], 0, sizeof(double) * G.gsize, h->stream));
    }
    return momentum_sums(h);
  }
  k_dep_trilinear<<<blocks_for(G.gsize), kThreads, 0, h->stream>>>(G, d, 0, h->dep[PSTEP_FIELD_C]);
  PSTEP_LAUNCHED(h);
  double *c1[1] = {h->dep[PSTEP_FIELD_C]};
  int rc = fold_fields(h, c1, 1, 0);  // the reference does not refresh C's ghosts
  if (rc) return rc;
  if (h->cfg.twc) {
    k_dep_face<0><<<blocks_for(G.gsize), kThreads, 0, h->stream>>>(G, d, h->dep[PSTEP_FIELD_RU_X]);
    PSTEP_LAUNCHED(h);
    k_dep_face<1><<<blocks_for(G.gsize), kThreads, 0, h->stream>>>(G, d, h->dep[PSTEP_FIELD_RU_Y]);
    PSTEP_LAUNCHED(h);
    k_dep_face<2><<<blocks_for(G.gsize), kThreads, 0, h->stream>>>(G, d, h->dep[PSTEP_FIELD_RU_Z]);
    PSTEP_LAUNCHED(h);
    double *ru[3] = {h->dep[PSTEP_FIELD_RU_X], h->dep[PSTEP_FIELD_RU_Y], h->dep[PSTEP_FIELD_RU_Z]};
    rc = fold_fields(h, ru, 3, 1);
    if (rc) return rc;
  } else {
    for (int q = PSTEP_FIELD_RU_X; q <= PSTEP_FIELD_RU_Z; ++q)
      PSTEP_CUDA(cudaMemsetAsync(h->dep[q], 0, sizeof(double) * G.gsize, h->stream));  // RHS_RU = 0 (grid.cpp:671)
  }
  return momentum_sums(h);
}

}  // namespace pstep
