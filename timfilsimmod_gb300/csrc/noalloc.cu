// noalloc.cu -- the segment-segment mobility product without any device
// allocation, for callers that cannot allocate.
//
// Some hosts of this code run the mobility product where cudaMalloc is not
// allowed or not wanted: a simulation driver that reserves all device memory
// up front for its own pool, a real-time loop that must not block on an
// allocation (cudaMalloc can synchronise the device), or code that runs
// inside another framework's stream capture. tfs_mss_noalloc serves them: the
// caller passes device pointers for the inputs and the output, and the only
// working memory -- the packed source records and the per-split partial sums
// of the tile kernel -- is the file-scope array below, which every GPU that
// loads this library holds until the process exits.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/tfs_gb300.h"
#include "tfs_kernels.h"

namespace tfs {
int fail(int code, const char *fmt, ...);
int cuda_fail(cudaError_t e, const char *what);
}  // namespace tfs

using namespace tfs;

namespace {

constexpr int kMaxSegs = TFS_NOALLOC_MAX_SEGS;
constexpr int kRecordDoubles = 10;   // FP64 segment record {x,y,z,f0..f5,0}
constexpr int kMaxSplitsNoalloc = 8; // partial sums kept for up to 8 source splits
constexpr size_t kRecordElems = (size_t)kRecordDoubles * kMaxSegs;
constexpr size_t kPartialElems = (size_t)kMaxSplitsNoalloc * 6 * kMaxSegs;

// 58 doubles per segment of capacity: 12 800 x 58 x 8 B = 5.9 MB per device.
__device__ __align__(256) double g_noalloc_scratch[kRecordElems + kPartialElems];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
double *g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch array on the current device, looked up once
// per device (host code may not use the array's name as a device address).
int scratch_for_current_device(double **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) return fail(TFS_EINVAL, "device ordinal %d out of range", dev);
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (g_scratch_ptr[dev] == nullptr) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(no-allocation scratch)");
    g_scratch_ptr[dev] = static_cast<double *>(p);
  }
  *out = g_scratch_ptr[dev];
  return TFS_OK;
}

}  // namespace

extern "C" int tfs_mss_noalloc(const double *x_segs, const double *f_segs, double *v_segs,
                               int num_segs, double mu, double a_seg, void *stream) {
  if (num_segs < 0) return fail(TFS_EINVAL, "negative segment count");
  if (num_segs > kMaxSegs)
    return fail(TFS_EINVAL,
                "num_segs %d exceeds the no-allocation limit of %d segments (use the solver API)",
                num_segs, kMaxSegs);
  if (!(mu > 0.0) || !(a_seg > 0.0)) return fail(TFS_EINVAL, "mu and a_seg must be positive");
  if (num_segs > 0 && (x_segs == nullptr || f_segs == nullptr || v_segs == nullptr))
    return fail(TFS_EINVAL, "null device pointer");
  double *scratch = nullptr;
  int rc = scratch_for_current_device(&scratch);
  if (rc != TFS_OK) return rc;
  if (num_segs == 0) return TFS_OK;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  double *records = scratch;
  double *partials = scratch + kRecordElems;
  cudaError_t e = launch_pack(0, 6, records, x_segs, f_segs, num_segs, nullptr, st);
  if (e != cudaSuccess) return cuda_fail(e, "pack kernel");
  TileArgs a{};
  a.x_tgt = x_segs;
  a.n_tgt = num_segs;
  a.a_tgt = a_seg;
  a.src_a = records;
  a.n_a = num_segs;
  a.a_a = a_seg;
  a.fp32 = 0;
  a.scale = 1.0 / (8.0 * 3.14159265358979323846264338327950288 * mu);
  a.out = v_segs;
  a.splits = kMaxSplitsNoalloc;  // the partial-sum capacity of the scratch array
  e = launch_tile(a, 6, 6, 0, TileTuning{0, 1}, partials, kPartialElems, OUT_ASSIGN, st);
  if (e != cudaSuccess) return cuda_fail(e, "segment-segment product");
  return TFS_OK;
}
