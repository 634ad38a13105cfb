// noalloc.cu -- points_affect_points for callers that cannot allocate device memory.
//
// Some callers cannot call cudaMalloc: code running inside a host framework that owns every
// device allocation (a pool allocator or memory budget that forbids side allocations),
// embedded or FFI callers (Fortran, plain C) that hand over finished device buffers and have
// no allocator of their own, and callers that must not trigger the implicit device
// synchronization an allocation can cause.  This entry point serves them: it allocates
// nothing.  Its scratch (work header, packed sources, split partials) is one file-scope
// device array of fixed size, reserved on every GPU that loads the library until the process
// exits.  The caller still passes all inputs and outputs as device pointers.
#include <algorithm>
#include <cstring>
#include <mutex>

#include "obs_context.h"
#include "p2p_dispatch.cuh"

namespace {

constexpr int kMaxSources = 262144;                                      // 1024 tiles of 256
constexpr size_t kHeaderBytes = 256;                                     // counter, meta, status
constexpr size_t kStatusOffset = 64;
constexpr size_t kSourceBytes = (size_t)kMaxSources * sizeof(float4);    // 4 MiB
constexpr size_t kPartialBytes = (size_t)12 << 20;                       // 12 MiB
constexpr size_t kScratchBytes = kHeaderBytes + kSourceBytes + kPartialBytes;

// The fixed scratch.  In host code this name is only a stand-in, not a device address: its
// device address comes from cudaGetSymbolAddress (below), once per device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_scratch_addr[kMaxDevices];
int g_num_sms[kMaxDevices];

// Device address of the scratch on the current device, looked up on the first call there.
int scratch_on_current_device(void** addr, int* num_sms) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return obs::cuda_status(e);
  if (dev < 0 || dev >= kMaxDevices) return OBS_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) return obs::cuda_status(e == cudaSuccess ? cudaErrorInvalidSymbol : e);
    int sms = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return obs::cuda_status(e);
    g_num_sms[dev] = sms;
    g_scratch_addr[dev] = p;
  }
  *addr = g_scratch_addr[dev];
  *num_sms = g_num_sms[dev];
  return OBS_OK;
}

}  // namespace

extern "C" int obs_points_affect_points_noalloc(void* cuda_stream, int core, int result, int accum, int flags,
                                                double fsx, double fsy,
                                                int ns, const float* sx, const float* sy, const float* sr,
                                                const float* ss,
                                                int nt, const float* tx, const float* ty, const float* tr,
                                                float* tu, float* tv,
                                                float* e0, float* e1, float* e2, float* e3) {
  using namespace obs;
  if (core < OBS_CORE_RM || core > OBS_CORE_COMPACT_EXP) return OBS_ERR_ARG;
  if (result < OBS_VELONLY || result > OBS_VELANDSHEAR) return OBS_ERR_ARG;
  if (accum != OBS_PLAIN_F32 && accum != OBS_COMPENSATED) return OBS_ERR_ARG;
  if (ns < 0 || nt < 0) return OBS_ERR_ARG;
  if (ns > kMaxSources) return OBS_ERR_SCRATCH_LIMIT;
  float* extra[4] = {e0, e1, e2, e3};
  const int nextra = result == OBS_VELANDGRAD ? 4 : (result == OBS_VELONLY ? 0 : 1);
  if (ns > 0 && (!sx || !sy || !ss || (core != OBS_CORE_SINGULAR && !sr))) return OBS_ERR_ARG;
  if (nt > 0 && (!tx || !ty || (result != OBS_PSIONLY && (!tu || !tv)))) return OBS_ERR_ARG;
  for (int k = 0; k < nextra; ++k)
    if (nt > 0 && !extra[k]) return OBS_ERR_ARG;
  if (ns == 0 || nt == 0) return OBS_OK;
  cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
  // the call ends by synchronizing its stream, which a stream capture does not allow
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone) return OBS_ERR_UNSUPPORTED;

  void* base = nullptr;
  int nsm = 0;
  int s = scratch_on_current_device(&base, &nsm);
  if (s) return s;
  const bool thick = tr != nullptr;
  const bool comp = accum == OBS_COMPENSATED;
  const int res = result;
  const int kcore = (res == RES_PSI) ? CORE_RM : core;

  // plan: same rule as the context path, then fewer splits until the partials fit
  int occ = 0;
  cudaError_t e = p2p_dispatch_any(core, thick, res, comp, nullptr, 0, st, &occ);
  if (e != cudaSuccess) return cuda_status(e);
  occ = std::max(occ, 1);
  const int slots = occ * nsm;
  const int tb = P2P_THREADS * p2p_tpt(res);
  const int ntb = (nt + tb - 1) / tb;
  const int nst = (ns + SRC_TILE - 1) / SRC_TILE;
  const int nc = p2p_ncomp(res);
  const size_t elem = comp ? sizeof(double) : sizeof(float);
  int nsplit = std::max(1, (24 * slots + ntb - 1) / ntb);
  nsplit = std::min(nsplit, std::max(1, std::min(nst / 2, 512)));
  const size_t fit = kPartialBytes / ((size_t)nc * (size_t)nt * elem);
  nsplit = std::max(1, std::min<int>(nsplit, (int)std::min<size_t>(fit, (size_t)nst)));
  const int tps = (nst + nsplit - 1) / nsplit;
  nsplit = (nst + tps - 1) / tps;

  char* scratch = static_cast<char*>(base);
  WorkHeader* h = reinterpret_cast<WorkHeader*>(scratch);
  int* status = reinterpret_cast<int*>(scratch + kStatusOffset);
  float4* src = reinterpret_cast<float4*>(scratch + kHeaderBytes);
  void* part = nsplit > 1 ? static_cast<void*>(scratch + kHeaderBytes + kSourceBytes) : nullptr;

  // the array keeps the previous call's contents: clear the counter, radius extrema, status
  e = cudaMemsetAsync(scratch, 0, kHeaderBytes, st);
  if (e != cudaSuccess) return cuda_status(e);
  e = p2p_launch_pack(sx, sy, sr, ss, ns, nst * SRC_TILE, kcore, src, h->meta, st);
  if (e == cudaSuccess && thick) e = p2p_launch_target_meta(tr, nt, h->meta, st);
  if (e != cudaSuccess) return cuda_status(e);

  P2PArgs a;
  std::memset(&a, 0, sizeof(a));
  a.src = src; a.nst = nst;
  a.tx = tx; a.ty = ty; a.tr = tr;
  a.nt = nt; a.ntb = ntb;
  a.nsplit = nsplit; a.tiles_per_split = tps; a.nitems = ntb * nsplit;
  a.counter = &h->counter; a.meta = h->meta; a.status = status;
  a.out[0] = tu; a.out[1] = tv;
  for (int k = 0; k < 4; ++k) a.out[2 + k] = extra[k];
  a.part = part;
  a.direct = nsplit == 1;
  a.finalize = (flags & OBS_FLAG_FINALIZE) ? 1 : 0;
  a.fsx = fsx; a.fsy = fsy;
  e = p2p_dispatch_any(core, thick, res, comp, &a, std::min(a.nitems, slots), st, nullptr);
  if (e == cudaSuccess && nsplit > 1) e = p2p_reduce(res, comp, a, st);
  if (e != cudaSuccess) return cuda_status(e);

  // report device-side failures of this call (bounded waits): read the status words
  int w[4] = {0, 0, 0, 0};
  e = cudaMemcpyAsync(w, status, sizeof(w), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_status(e);
  if (w[0] & DEV_ERR_TIMEOUT) return OBS_ERR_TIMEOUT;
  if (w[0]) return OBS_ERR_CUDA;
  return OBS_OK;
}
