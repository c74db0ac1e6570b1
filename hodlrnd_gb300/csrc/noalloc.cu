// hodlr_aca_block_noalloc: compress one block with the engine's ACA kernel
// without allocating any device memory.
//
// Who needs it: code that cannot call cudaMalloc at the point where it wants a
// block compressed -- a host framework that owns all device memory through its
// own pool, a latency-critical loop where cudaMalloc's implicit device
// synchronisation is unacceptable, or code running while another component
// forbids allocation.  Such a caller provides the inputs (points, index lists)
// and the output buffer; the ACA's bookkeeping -- the bitmaps of remaining
// rows and columns, the lists of used pivots, the block descriptor and the
// result -- lives in the file-scope array below instead of in memory the engine
// would otherwise allocate per build.
//
// The array is a fixed ~136 KB and every GPU that loads this library keeps it
// until the process exits.  All calls share it: a call rewrites what it needs
// (the kernel re-initialises the bitmaps, the descriptor and the index lists
// are copied in, the result slot is cleared), so nothing carries over from the
// previous call, but two calls whose work overlaps on the GPU (different
// streams, or different host threads) race on it and must be serialised by
// the caller.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <string>

#include "../../include/hodlrnd.h"
#include "aca.h"

namespace hodlr {
void set_thread_error(const std::string& msg);  // engine.cu: hodlr_last_error(NULL)
}

namespace {

using hodlr::AcaArgs;
using hodlr::AcaBlockDesc;
using hodlr::AcaOut;

constexpr int kMaxPoints = HODLR_NOALLOC_MAX_POINTS;
constexpr int kMaxCap = HODLR_NOALLOC_MAX_RANK;

struct Scratch {
  int32_t lmap[2 * kMaxPoints];        // row point indices, then column point indices
  uint32_t bits[2 * (kMaxPoints / 32)];  // remaining rows, remaining columns
  int32_t lists[2 * (kMaxCap + 2)];    // used rows, used columns
  AcaBlockDesc desc;
  AcaOut out;
  int32_t team[4];                     // the launch's team list: {0}
};

static __device__ __align__(256) unsigned char g_noalloc_scratch[sizeof(Scratch)];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_addr[kMaxDevices] = {};
void* g_ctx[kMaxDevices] = {};  // the context the address belongs to

int fail(int code, const std::string& msg) {
  hodlr::set_thread_error(msg);
  return code;
}

// The current context of the calling thread (driver cuCtxGetCurrent, reached
// through the runtime so that the library needs no link to libcuda); null
// when it cannot be queried.
void* current_context() {
  using GetCtx = int (*)(void**);
  static GetCtx fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      f = nullptr;
    return reinterpret_cast<GetCtx>(f);
  }();
  void* c = nullptr;
  if (!fn || fn(&c) != 0) return nullptr;
  return c;
}

// Device address of the scratch array on the current device.  It is looked
// up (cudaGetSymbolAddress) by the first call on a device and again whenever
// the device's context has changed since (after cudaDeviceReset the module is
// loaded anew, possibly elsewhere); a lookup must not happen inside a stream
// capture.
int scratch_address(Scratch** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(HODLR_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return fail(HODLR_ERR_INVALID, "device ordinal beyond the supported range");
  // null before the runtime has made the device's context current: the
  // lookup below does that, and the context is read again after it
  void* ctx = current_context();
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_addr[dev] || !ctx || ctx != g_ctx[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return fail(HODLR_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    g_addr[dev] = p;
    g_ctx[dev] = current_context();
  }
  *out = static_cast<Scratch*>(g_addr[dev]);
  return HODLR_OK;
}

}  // namespace

extern "C" int hodlr_aca_block_noalloc(const double* d_points, int64_t ld, int32_t ndim, const int32_t* d_rows,
                                       int32_t m, const int32_t* d_cols, int32_t n, const hodlr_kernel_desc* kernel,
                                       double eps_aca, uint64_t seed, int32_t cap, double* d_factors, int32_t* rank,
                                       int32_t* flags, void* stream) {
  if (!d_points || !d_rows || !d_cols || !kernel || !d_factors || !rank || !flags)
    return fail(HODLR_ERR_INVALID, "hodlr_aca_block_noalloc: null argument");
  if (ndim < 1 || ndim > 8) return fail(HODLR_ERR_INVALID, "hodlr_aca_block_noalloc: ndim must be in 1..8");
  if (m < 1 || n < 1 || m > kMaxPoints || n > kMaxPoints)
    return fail(HODLR_ERR_INVALID, "hodlr_aca_block_noalloc: m and n must be in 1.." +
                                       std::to_string(kMaxPoints) + " (the size of the static scratch)");
  if (cap < 1 || cap > kMaxCap)
    return fail(HODLR_ERR_INVALID,
                "hodlr_aca_block_noalloc: cap must be in 1.." + std::to_string(kMaxCap) + " columns");
  if (ld < 1) return fail(HODLR_ERR_INVALID, "hodlr_aca_block_noalloc: ld must be positive");
  if (!(eps_aca > 0.0) || !(eps_aca < 1.0))
    return fail(HODLR_ERR_INVALID, "hodlr_aca_block_noalloc: eps_aca must be in (0, 1)");
  if (kernel->kind < HODLR_KERNEL_INV_R || kernel->kind > HODLR_KERNEL_EXP_NEG_R)
    return fail(HODLR_ERR_INVALID, "hodlr_aca_block_noalloc: unknown kernel kind");
  Scratch* s = nullptr;
  int rc = scratch_address(&s);
  if (rc != HODLR_OK) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);

  AcaBlockDesc desc;
  std::memset(&desc, 0, sizeof(desc));
  desc.t_map = 0;
  desc.s_map = m;
  desc.m = m;
  desc.n = n;
  desc.cap = cap;
  desc.ws = 0;
  desc.bits = 0;
  desc.lists = 0;
  desc.seed = seed;
  const int32_t team[4] = {0, 0, 0, 0};
  cudaError_t e;
  if ((e = cudaMemcpyAsync(s->lmap, d_rows, sizeof(int32_t) * size_t(m), cudaMemcpyDeviceToDevice, st)) ||
      (e = cudaMemcpyAsync(s->lmap + m, d_cols, sizeof(int32_t) * size_t(n), cudaMemcpyDeviceToDevice, st)) ||
      (e = cudaMemcpyAsync(&s->desc, &desc, sizeof(desc), cudaMemcpyHostToDevice, st)) ||
      (e = cudaMemcpyAsync(s->team, team, sizeof(team), cudaMemcpyHostToDevice, st)) ||
      (e = cudaMemsetAsync(&s->out, 0, sizeof(AcaOut), st)))
    return fail(HODLR_ERR_CUDA, std::string("hodlr_aca_block_noalloc: staging: ") + cudaGetErrorString(e));

  AcaArgs a;
  a.lmap = s->lmap;
  a.P = hodlr::PointsDev{d_points, ld};
  a.K = hodlr::KernelDev{kernel->kind, kernel->scale, kernel->diag};
  a.tol = eps_aca;
  a.blocks = &s->desc;
  a.ws = d_factors;  // U (m x cap) then V (n x cap): the caller's output buffer
  a.bits = s->bits;
  a.lists = s->lists;
  a.out = &s->out;
  a.arena_off = 0;
  a.arena_size = 0;
  a.arena_used = nullptr;  // no growth: a block that needs more than cap columns reports it
  a.queue = nullptr;
  a.max_ctas = 0;
  // the team hodlr_build gives a block of this size (the team size sets the
  // summation order of the stopping rule's norms)
  hodlr::AcaLists al;
  for (int k = 0; k < hodlr::kAcaTeamKinds; k++) {
    al.list[k] = s->team;
    al.n[k] = 0;
  }
  al.n[hodlr::aca_team(m, n)] = 1;
  e = hodlr::launch_aca(ndim, a, al, st);
  if (e != cudaSuccess)
    return fail(HODLR_ERR_CUDA, std::string("hodlr_aca_block_noalloc: launch: ") + cudaGetErrorString(e));
  AcaOut out;
  if ((e = cudaMemcpyAsync(&out, &s->out, sizeof(out), cudaMemcpyDeviceToHost, st)) ||
      (e = cudaStreamSynchronize(st)))
    return fail(HODLR_ERR_CUDA, std::string("hodlr_aca_block_noalloc: ") + cudaGetErrorString(e));
  *rank = out.rank;
  *flags = out.flags;
  return HODLR_OK;
}
