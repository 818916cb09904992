// The coarse step (exact query x centroid distances, then the nprobe nearest
// lists per query) for callers that cannot allocate device memory.
//
// katoann_gpu_coarse needs nq x nlist floats of scratch for the distance
// matrix, which its caller allocates. Some callers cannot: a host process
// that embeds this library as a plug-in may hand every byte of device memory
// to its own allocator and forbid any other allocation, and a latency-bound
// serving loop cannot afford cudaMalloc, which can synchronise the whole
// device. katoann_gpu_coarse_noalloc keeps that scratch in a static device
// array instead, sized for at most kNoAllocMaxDists distances (nq * nlist
// <= 1,048,576, i.e. 4 MiB); every GPU that loads this library holds the array
// until the process exits. The caller still passes the inputs and the output.
//
// Set-up: the first call on a device looks up the array's device address with
// cudaGetSymbolAddress while that device is current (once per device, under a
// lock). Make that first call before capturing a stream into a CUDA graph.
// All calls share the one array and it keeps the last call's contents; every
// call overwrites the part it uses before reading it, so nothing needs
// clearing. Calls whose work overlaps on the GPU (different streams, or
// different host threads) race on the array: serialise them.
#include <mutex>

#include "kcommon.cuh"

namespace kato {
int sq16_tiles(const uint8_t *qhi, const uint8_t *qlo, const uint8_t *xhi, const uint8_t *xlo,
               const int64_t *qn, const int64_t *xn, double step_sq, uint32_t m, uint32_t n,
               uint32_t dims, uint32_t qstride, uint32_t xstride, float *out, bool full,
               cudaStream_t st);
int select_topp(const float *dists, uint32_t nq, uint32_t n, uint32_t p, uint32_t *probed,
                unsigned long long *tie_count, cudaStream_t st);
}  // namespace kato

namespace {

constexpr size_t kNoAllocMaxDists = size_t(1) << 20;  // nq * nlist distances (4 MiB)
constexpr int kMaxDevices = 64;

// The scratch of the distance matrix. Host code must not use this name as an
// address: it resolves the device address with cudaGetSymbolAddress.
static __device__ __align__(256) float g_coarse_scratch[kNoAllocMaxDists];

std::mutex g_scratch_mu;
float *g_scratch_addr[kMaxDevices] = {};

int scratch_address(float **out) {
  int dev = 0;
  KATO_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return kato::invalid("device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_addr[dev]) {
    void *p = nullptr;
    KATO_CUDA(cudaGetSymbolAddress(&p, g_coarse_scratch));
    g_scratch_addr[dev] = static_cast<float *>(p);
  }
  *out = g_scratch_addr[dev];
  return KATO_OK;
}

}  // namespace

extern "C" int katoann_gpu_coarse_noalloc(const katoann_gpu_index *ix, const uint8_t *d_qhi,
                                          const uint8_t *d_qlo, const int64_t *d_qnorm,
                                          uint32_t nq, uint32_t nprobe, uint32_t *d_probed,
                                          katoann_stream_t stream) {
  if (!ix) return kato::invalid("null index");
  if (nprobe == 0 || nprobe > ix->nlist) return kato::invalid("need k >= 1 and 1 <= nprobe <= nlist");
  if (static_cast<uint64_t>(nq) * ix->nlist > kNoAllocMaxDists)
    return kato::invalid("katoann_gpu_coarse_noalloc: nq * nlist exceeds its static scratch of "
                         "1048576 distances; split the batch or use katoann_gpu_coarse");
  if (nq == 0) return KATO_OK;
  float *scratch = nullptr;
  int rc = scratch_address(&scratch);
  if (rc) return rc;
  const cudaStream_t st = kato::as_stream(stream);
  rc = kato::sq16_tiles(d_qhi, d_qlo, ix->d_chi, ix->d_clo, d_qnorm, ix->d_cnorm, ix->step_sq, nq,
                        ix->nlist, ix->dc, ix->dc, ix->dc, scratch, true, st);
  if (rc) return rc;
  return kato::select_topp(scratch, nq, ix->nlist, nprobe, d_probed, nullptr, st);
}
