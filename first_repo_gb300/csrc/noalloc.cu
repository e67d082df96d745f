// pstep_field_mean_noalloc: the interior mean of a ghosted field (the same
// quantity as pstep_energy_mean) without any device allocation.
//
// For callers that cannot call cudaMalloc: code that records its work into a
// CUDA graph during stream capture (allocation is not allowed while capturing),
// applications that hand all device memory to their own pool, and loops that
// must not synchronise the device (cudaMalloc/cudaFree do). The reduction's
// scratch -- one fp64 partial sum per (j, k) row of the interior -- lives in a
// file-scope device array of fixed size, which every GPU that loads this
// library keeps until the process exits.
#include <mutex>
#include "pstep_internal.cuh"

namespace {

// Maximum number of interior rows ny * nz (e.g. 1024 x 1024): 8 MiB of scratch.
constexpr int64_t kNoallocMaxRows = 1 << 20;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_row_sums[kNoallocMaxRows];

double *g_row_addr[kMaxDevices] = {nullptr};
std::mutex g_row_mutex;
// one message buffer per calling thread, so that two threads failing at once
// each read their own message
thread_local char g_noalloc_err[256] = "";

// one warp per row: fixed-order sum of the row's interior cells
__global__ void k_row_sums(const double *__restrict__ f, int nx, int ny, int nz, double *__restrict__ rows) {
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int64_t nrows = (int64_t)ny * nz;
  if (warp >= nrows) return;
  const int j = (int)(warp % ny) + 1, k = (int)(warp / ny) + 1;
  const int64_t gx = nx + 2, gy = ny + 2;
  const double *row = f + ((int64_t)k * gy + j) * gx;
  double s = 0.0;
  for (int i = lane + 1; i <= nx; i += 32) s += row[i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if (lane == 0) rows[warp] = s;
}

// one block: fixed-order sum of the row sums, times 1/(nx*ny*nz)
__global__ void k_rows_total(const double *__restrict__ rows, int64_t nrows, double inv, double *__restrict__ out) {
  __shared__ double sm[256];
  double s = 0.0;
  for (int64_t r = threadIdx.x; r < nrows; r += blockDim.x) s += rows[r];
  sm[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sm[threadIdx.x] += sm[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sm[0] * inv;
}

}  // namespace

extern "C" const char *pstep_noalloc_last_error(void) { return g_noalloc_err; }

extern "C" int pstep_field_mean_noalloc(const double *field, int32_t nx, int32_t ny, int32_t nz, double *out,
                                        void *stream) {
  if (!field || !out || nx < 1 || ny < 1 || nz < 1) {
    snprintf(g_noalloc_err, sizeof g_noalloc_err, "invalid argument");
    return PSTEP_ERR_ARG;
  }
  const int64_t nrows = (int64_t)ny * nz;
  if (nrows > kNoallocMaxRows) {
    snprintf(g_noalloc_err, sizeof g_noalloc_err,
             "ny*nz = %lld interior rows exceeds the fixed scratch of %lld rows", (long long)nrows,
             (long long)kNoallocMaxRows);
    return PSTEP_ERR_CAPACITY;
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    snprintf(g_noalloc_err, sizeof g_noalloc_err, "no usable current CUDA device");
    return PSTEP_ERR_CUDA;
  }
  cudaStream_t s = (cudaStream_t)stream;
  double *rows = nullptr;
  {
    // set-up, once per device, with that device current: the device address of the scratch array
    std::lock_guard<std::mutex> lock(g_row_mutex);
    if (!g_row_addr[dev]) {
      // the look-up is not a stream operation and may end a capture in progress: refuse
      // cleanly instead, the caller makes one call on this device before capturing
      cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
      if (cudaStreamIsCapturing(s, &cs) != cudaSuccess) {
        cudaGetLastError();
        snprintf(g_noalloc_err, sizeof g_noalloc_err, "cudaStreamIsCapturing failed");
        return PSTEP_ERR_CUDA;
      }
      if (cs != cudaStreamCaptureStatusNone) {
        snprintf(g_noalloc_err, sizeof g_noalloc_err,
                 "first call on device %d made while its stream is being captured: make one call before capture",
                 dev);
        return PSTEP_ERR_STATE;
      }
      cudaError_t e = cudaGetSymbolAddress((void **)&g_row_addr[dev], g_row_sums);
      if (e != cudaSuccess) {
        g_row_addr[dev] = nullptr;
        cudaGetLastError();
        snprintf(g_noalloc_err, sizeof g_noalloc_err, "cudaGetSymbolAddress: %s", cudaGetErrorString(e));
        return PSTEP_ERR_CUDA;
      }
    }
    rows = g_row_addr[dev];
  }
  const int threads = 256;
  const int64_t blocks = (nrows * 32 + threads - 1) / threads;
  k_row_sums<<<(unsigned)blocks, threads, 0, s>>>(field, nx, ny, nz, rows);
  k_rows_total<<<1, 256, 0, s>>>(rows, nrows, 1.0 / ((double)nx * ny * nz), out);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    snprintf(g_noalloc_err, sizeof g_noalloc_err, "launch: %s", cudaGetErrorString(e));
    return PSTEP_ERR_CUDA;
  }
  return PSTEP_OK;
}
