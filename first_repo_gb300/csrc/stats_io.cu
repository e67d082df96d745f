// Diagnostics reductions and snapshot files of the particle state.
//
//   particle::NP_TOT, max, Balance_Index, find_tag      particle.cpp:662-741
//   tensor0::max, min, sum/mean of a deposited field    tensor0.cpp:418-503
//     (what the reference's statistics output takes of C, grid.cpp:715-735)
//   particle::Store_All / Load_All                      particle.cpp:867-1025
//
// Maxima and minima are exact in any order. The field mean is a fixed-order
// tree sum (coalesced rows per block, then one block) divided by n^3 as the
// reference divides by size_tot(); the reference sums in its i-j-k loop order,
// so the mean can differ from it in the last bits.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#include <algorithm>

#include "pstep_internal.cuh"

namespace pstep {
int f32_positions(pstep_ctx *h, const int32_t *idx, int32_t n, double *xyz);  // stage_f32.cu
}

namespace {
using namespace pstep;

constexpr int kStatBlocks = 1024;

int fail_io(pstep_ctx *h, int code, const std::string &msg) {
  snprintf(h->err, sizeof h->err, "%s", msg.c_str());
  return code;
}

template <typename T>
int dalloc_tmp(pstep_ctx *h, T *&p, size_t count) {
  p = nullptr;
  cudaError_t e = cudaMalloc((void **)&p, sizeof(T) * (count ? count : 1));
  if (e != cudaSuccess) {
    p = nullptr;
    cudaGetLastError();
    snprintf(h->err, sizeof h->err, "cudaMalloc: %s", cudaGetErrorString(e));
    return PSTEP_ERR_NOMEM;
  }
  return PSTEP_OK;
}

// block reductions of three values (max, min, sum) over kThreads threads
__device__ void block_reduce3(double &mx, double &mn, double &sm) {
  __shared__ double s_mx[kThreads], s_mn[kThreads], s_sm[kThreads];
  s_mx[threadIdx.x] = mx;
  s_mn[threadIdx.x] = mn;
  s_sm[threadIdx.x] = sm;
  __syncthreads();
  for (int o = kThreads / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) {
      s_mx[threadIdx.x] = fmax(s_mx[threadIdx.x], s_mx[threadIdx.x + o]);
      s_mn[threadIdx.x] = fmin(s_mn[threadIdx.x], s_mn[threadIdx.x + o]);
      s_sm[threadIdx.x] += s_sm[threadIdx.x + o];
    }
    __syncthreads();
  }
  mx = s_mx[0];
  mn = s_mn[0];
  sm = s_sm[0];
}

// largest of a[0 .. n): per-block partials
__global__ void k_max_partial(const double *__restrict__ a, int64_t n, double *__restrict__ part) {
  double mx = -INFINITY, mn = 0.0, sm = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    mx = fmax(mx, a[i]);
  block_reduce3(mx, mn, sm);
  if (threadIdx.x == 0) part[blockIdx.x] = mx;
}

// interior maximum, minimum and sum of a ghosted field: rows (j,k) over blocks, the
// i loop over threads (coalesced, fixed order)
__global__ void k_field_partial(Geom G, const double *__restrict__ f, double *__restrict__ part) {
  double mx = -INFINITY, mn = INFINITY, sm = 0.0;
  const long long rows = (long long)G.n[1] * G.n[2];
  for (long long r = blockIdx.x; r < rows; r += gridDim.x) {
    const int j = (int)(r % G.n[1]) + 1, k = (int)(r / G.n[1]) + 1;
    const double *row = f + glin(G, 0, j, k);
    for (int i = threadIdx.x + 1; i <= G.n[0]; i += blockDim.x) {
      const double v = row[i];
      mx = fmax(mx, v);
      mn = fmin(mn, v);
      sm += v;
    }
  }
  block_reduce3(mx, mn, sm);
  if (threadIdx.x == 0) {
    part[3 * blockIdx.x] = mx;
    part[3 * blockIdx.x + 1] = mn;
    part[3 * blockIdx.x + 2] = sm;
  }
}

// stride 1: part holds maxima only (out[0]); stride 3: (max, min, sum) triples
__global__ void k_stat_final(const double *__restrict__ part, int np, int stride, double *__restrict__ out) {
  double mx = -INFINITY, mn = INFINITY, sm = 0.0;
  for (int i = threadIdx.x; i < np; i += kThreads) {
    mx = fmax(mx, part[stride * i]);
    if (stride == 3) {
      mn = fmin(mn, part[3 * i + 1]);
      sm += part[3 * i + 2];
    }
  }
  block_reduce3(mx, mn, sm);
  if (threadIdx.x == 0) {
    out[0] = mx;
    out[1] = mn;
    out[2] = sm;
  }
}

// storage index of the particle carrying each sought id (sorted ids, -1 when absent;
// the smallest index if an id repeats, as find_tag's loop finds the first)
__global__ void k_find_tags(const int32_t *__restrict__ flag, int64_t n, const int32_t *__restrict__ tags, int nt,
                            int32_t *__restrict__ idx) {
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    const int32_t v = flag[p];
    int lo = 0, hi = nt;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (tags[mid] < v) lo = mid + 1; else hi = mid;
    }
    if (lo < nt && tags[lo] == v) atomicMin(&idx[lo], (int32_t)p);
  }
}

__global__ void k_fill_i32(int32_t *a, int n, int32_t v) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) a[i] = v;
}

__global__ void k_positions64(const double *__restrict__ x, const double *__restrict__ y,
                              const double *__restrict__ z, const int32_t *__restrict__ idx, int32_t n,
                              double *__restrict__ xyz) {
  const int32_t i = (int32_t)(blockIdx.x * blockDim.x + threadIdx.x);
  if (i >= n) return;
  const int32_t p = idx[i];
  if (p < 0) return;
  xyz[3 * i] = x[p];
  xyz[3 * i + 1] = y[p];
  xyz[3 * i + 2] = z[p];
}

const char *const kSnapNames[8] = {"Part_x", "Part_y", "Part_z", "Part_u", "Part_v", "Part_w", "Part_T", "Part_flag"};
const int kSnapIds[8] = {PSTEP_X, PSTEP_Y, PSTEP_Z, PSTEP_U, PSTEP_V, PSTEP_W, PSTEP_T, PSTEP_FLAG};

}  // namespace

extern "C" {

int pstep_np_tot(pstep_handle h, int64_t *out) {
  if (!h || !out) return PSTEP_ERR_ARG;
  *out = h->np;
  return PSTEP_OK;
}

int pstep_balance_index(pstep_handle h, double *out) {
  if (!h || !out) return PSTEP_ERR_ARG;
  const double np = (double)h->np;  // one rank: the largest and the smallest count are this one
  *out = np / np;
  return PSTEP_OK;
}

int pstep_max(pstep_handle h, int id, double *out) {
  if (!h || !out || id < 0 || id >= PSTEP_NUM_ARRAYS || id == PSTEP_FLAG) return PSTEP_ERR_ARG;
  const int64_t n = h->np;
  if (n == 0) {
    *out = -1e9;  // particle.cpp:674
    return PSTEP_OK;
  }
  {
    // the last stage gathers max u and max ug in its epilogue
    const int fr = h->f32 ? f32_fused_max(h, id, out) : f64_fused_max(h, id, out);
    if (fr != -1) return fr;
  }
  double *vals = nullptr, *part = nullptr;
  int rc = dalloc_tmp(h, vals, (size_t)n);
  if (!rc) rc = dalloc_tmp(h, part, kStatBlocks + 3);
  if (!rc) rc = pstep_get_particle_array(h, id, vals, 1);
  if (!rc) {
    k_max_partial<<<kStatBlocks, kThreads, 0, h->stream>>>(vals, n, part);
    k_stat_final<<<1, kThreads, 0, h->stream>>>(part, kStatBlocks, 1, part + kStatBlocks);
    h->launches += 2;
    cudaError_t e = cudaMemcpyAsync(out, part + kStatBlocks, sizeof(double), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) rc = fail_io(h, PSTEP_ERR_CUDA, std::string("max: ") + cudaGetErrorString(e));
  }
  cudaFree(vals);
  cudaFree(part);
  return rc;
}

int pstep_field_stats(pstep_handle h, int field, double *max, double *min, double *mean) {
  if (!h || field < 0 || field >= PSTEP_NUM_FIELDS) return PSTEP_ERR_ARG;
  const Geom &G = h->geom;
  if (h->f32) {
    // the FP32 form's last-stage deposit gathers these in its flush (exact integer max,
    // min, sum); after any other deposit a pass below
    double r[3] = {0, 0, 0};
    const int fr = f32_field_stats(h, field, r);
    if (fr == PSTEP_OK) {
      if (max) *max = r[0];
      if (min) *min = r[1];
      if (mean) *mean = r[2] / (double)((long long)G.n[0] * G.n[1] * G.n[2]);
      return PSTEP_OK;
    }
    if (fr != -1) return fr;
  }
  double *part = nullptr;
  int rc = dalloc_tmp(h, part, 3 * kStatBlocks + 3);
  if (rc) return rc;
  k_field_partial<<<kStatBlocks, kThreads, 0, h->stream>>>(G, h->dep[field], part);
  k_stat_final<<<1, kThreads, 0, h->stream>>>(part, kStatBlocks, 3, part + 3 * kStatBlocks);
  h->launches += 2;
  double r[3] = {0, 0, 0};
  cudaError_t e = cudaMemcpyAsync(r, part + 3 * kStatBlocks, sizeof r, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  cudaFree(part);
  if (e != cudaSuccess) return fail_io(h, PSTEP_ERR_CUDA, std::string("field stats: ") + cudaGetErrorString(e));
  if (max) *max = r[0];
  if (min) *min = r[1];
  // tensor0::mean: sum() / size_tot() (an int), tensor0.cpp:431-435
  if (mean) *mean = r[2] / (double)((long long)G.n[0] * G.n[1] * G.n[2]);
  return PSTEP_OK;
}

int pstep_find_tags(pstep_handle h, const int32_t *tags, int32_t n, double *xyz, int32_t *found) {
  if (!h || n < 0 || (n > 0 && (!tags || !xyz || !found))) return PSTEP_ERR_ARG;
  if (n == 0) return PSTEP_OK;
  if (!h->s.flag && h->np > 0) return fail_io(h, PSTEP_ERR_STATE, "no particles uploaded");
  // sorted distinct ids on the device, each remembering where the caller listed it
  std::vector<std::pair<int32_t, int32_t>> order((size_t)n);
  for (int32_t i = 0; i < n; ++i) order[(size_t)i] = {tags[i], i};
  std::sort(order.begin(), order.end());
  std::vector<int32_t> sorted((size_t)n);
  for (int32_t i = 0; i < n; ++i) sorted[(size_t)i] = order[(size_t)i].first;
  int32_t *d_tags = nullptr, *d_idx = nullptr;
  double *d_xyz = nullptr;
  int rc = dalloc_tmp(h, d_tags, (size_t)n);
  if (!rc) rc = dalloc_tmp(h, d_idx, (size_t)n);
  if (!rc) rc = dalloc_tmp(h, d_xyz, 3 * (size_t)n);
  std::vector<int32_t> idx((size_t)n, -1);
  std::vector<double> pos(3 * (size_t)n, 0.0);
  if (!rc) {
    cudaError_t e = cudaMemcpyAsync(d_tags, sorted.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, h->stream);
    k_fill_i32<<<(n + kThreads - 1) / kThreads, kThreads, 0, h->stream>>>(d_idx, n, INT32_MAX);
    if (h->np > 0)
      k_find_tags<<<kStatBlocks, kThreads, 0, h->stream>>>(h->s.flag, h->np, d_tags, n, d_idx);
    h->launches += h->np > 0 ? 2 : 1;
    if (e == cudaSuccess) e = cudaMemcpyAsync(idx.data(), d_idx, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) rc = fail_io(h, PSTEP_ERR_CUDA, std::string("find_tags: ") + cudaGetErrorString(e));
  }
  if (!rc) {
    for (auto &v : idx)
      if (v == INT32_MAX) v = -1;
    // an id asked for more than once: only its first sorted copy was searched for
    for (int32_t q = 1; q < n; ++q)
      if (sorted[(size_t)q] == sorted[(size_t)q - 1]) idx[(size_t)q] = idx[(size_t)q - 1];
    cudaError_t e = cudaMemcpyAsync(d_idx, idx.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, h->stream);
    if (e != cudaSuccess) rc = fail_io(h, PSTEP_ERR_CUDA, std::string("find_tags: ") + cudaGetErrorString(e));
  }
  if (!rc) {
    if (h->f32) {
      rc = f32_positions(h, d_idx, n, d_xyz);
    } else {
      k_positions64<<<(n + kThreads - 1) / kThreads, kThreads, 0, h->stream>>>(h->s.base[0], h->s.base[1],
                                                                                h->s.base[2], d_idx, n, d_xyz);
      h->launches += 1;
    }
  }
  if (!rc) {
    cudaError_t e = cudaMemcpyAsync(pos.data(), d_xyz, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) rc = fail_io(h, PSTEP_ERR_CUDA, std::string("find_tags: ") + cudaGetErrorString(e));
  }
  if (!rc) {
    for (int32_t s = 0; s < n; ++s) {
      const int32_t i = order[(size_t)s].second;
      found[i] = idx[(size_t)s] >= 0 ? 1 : 0;
      if (found[i])
        for (int d = 0; d < 3; ++d) xyz[3 * i + d] = pos[3 * (size_t)s + d];
    }
  }
  cudaFree(d_tags);
  cudaFree(d_idx);
  cudaFree(d_xyz);
  return rc;
}

int pstep_store_all(pstep_handle h, const char *data_dir, int num_ts) {
  if (!h || !data_dir) return PSTEP_ERR_ARG;
  const int64_t n = h->np;
  void *buf = nullptr;
  if (cudaMallocHost(&buf, sizeof(double) * (size_t)(n > 0 ? n : 1)) != cudaSuccess) {
    cudaGetLastError();
    return fail_io(h, PSTEP_ERR_NOMEM, "store_all: pinned host buffer");
  }
  int rc = PSTEP_OK;
  for (int q = 0; q < 8 && !rc; ++q) {
    const std::string path = std::string(data_dir) + kSnapNames[q] + "_" + std::to_string(num_ts) + ".bin";
    const size_t elem = q == 7 ? sizeof(int32_t) : sizeof(double);
    if (n > 0) rc = pstep_get_particle_array(h, kSnapIds[q], buf, 0);
    if (rc) break;
    FILE *f = fopen(path.c_str(), "wbx");  // MPI_MODE_CREATE | MPI_MODE_EXCL: never overwrite
    if (!f) {
      rc = fail_io(h, PSTEP_ERR_IO, "store_all: cannot create " + path + " (exists, or no such directory)");
      break;
    }
    const size_t wrote = n > 0 ? fwrite(buf, elem, (size_t)n, f) : 0;
    if (fclose(f) != 0 || wrote != (size_t)n) rc = fail_io(h, PSTEP_ERR_IO, "store_all: short write to " + path);
  }
  cudaFreeHost(buf);
  return rc;
}

int pstep_load_all(pstep_handle h, const char *dir, int64_t n0, int box) {
  if (!h || !dir || n0 < 0) return PSTEP_ERR_ARG;
  if (n0 > h->cap) return fail_io(h, PSTEP_ERR_CAPACITY, "load_all: more particles than capacity");
  std::vector<void *> bufs(8, nullptr);
  int rc = PSTEP_OK;
  for (int q = 0; q < 8 && !rc; ++q) {
    const size_t elem = q == 7 ? sizeof(int32_t) : sizeof(double);
    if (cudaMallocHost(&bufs[(size_t)q], elem * (size_t)(n0 > 0 ? n0 : 1)) != cudaSuccess) {
      cudaGetLastError();
      rc = fail_io(h, PSTEP_ERR_NOMEM, "load_all: pinned host buffer");
      break;
    }
    // particle.cpp:1000-1025: Restart_<name>.bin, the IO duct's names with _IO
    const std::string path = std::string(dir) + "Restart_" + kSnapNames[q] + (box ? "" : "_IO") + ".bin";
    FILE *f = fopen(path.c_str(), "rb");
    if (!f) {
      rc = fail_io(h, PSTEP_ERR_IO, "load_all: cannot open " + path);
      break;
    }
    const size_t got = n0 > 0 ? fread(bufs[(size_t)q], elem, (size_t)n0, f) : 0;
    fclose(f);
    if (got != (size_t)n0) rc = fail_io(h, PSTEP_ERR_IO, "load_all: short file " + path);
  }
  if (!rc) {
    const double *a[7];
    for (int q = 0; q < 7; ++q) a[q] = (const double *)bufs[(size_t)q];
    rc = pstep_upload_particles(h, n0, a[0], a[1], a[2], a[3], a[4], a[5], a[6], (const int32_t *)bufs[7], 0);
  }
  for (void *b : bufs)
    if (b) cudaFreeHost(b);
  return rc;
}

}  // extern "C"
