// Host runtime: errors, device properties, workspace, launch counting, and
// the small C-ABI helpers (perks_last_error, perks_status_string, ...).
#include "runtime.cuh"
#include "ptx.cuh"
#include <mutex>
#include <vector>

namespace perks {

static thread_local std::string g_last_error;
static thread_local long long g_launches = 0;
static long long g_ws_allocs = 0;  // cudaMalloc calls made by workspace() (guarded by g_mu)

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  std::string m = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
  if (e == cudaErrorMemoryAllocation) return fail(PERKS_ERR_OOM, m);
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return fail(PERKS_ERR_NO_DEVICE, m);
  if (e == cudaErrorCooperativeLaunchTooLarge) return fail(PERKS_ERR_LAUNCH, m);
  return fail(PERKS_ERR_CUDA, m);
}

static std::mutex g_mu;
static std::vector<DeviceInfo> g_devs;

const DeviceInfo* device_info() {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    cuda_fail(e, "cudaGetDevice");
    return nullptr;
  }
  std::lock_guard<std::mutex> lk(g_mu);
  if ((int)g_devs.size() <= dev) g_devs.resize(dev + 1);
  DeviceInfo& d = g_devs[dev];
  if (d.device < 0) {
    cudaDeviceProp prop;
    e = cudaGetDeviceProperties(&prop, dev);
    if (e != cudaSuccess) {
      cuda_fail(e, "cudaGetDeviceProperties");
      return nullptr;
    }
    if (prop.major < 10) {
      fail(PERKS_ERR_UNSUPPORTED, "this library is built for sm_103a (GB300); device is sm_" +
                                      std::to_string(prop.major) + std::to_string(prop.minor));
      return nullptr;
    }
    d.sms = prop.multiProcessorCount;
    d.smem_optin = prop.sharedMemPerBlockOptin;
    d.coop = prop.cooperativeLaunch;
    d.device = dev;
  }
  return &d;
}

struct WsEntry {
  void* ptr = nullptr;
  size_t bytes = 0;
};
static std::vector<std::vector<WsEntry>> g_ws;  // [device][slot]

void* workspace(WorkSlot slot, size_t bytes, int* status) {
  *status = PERKS_OK;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    *status = cuda_fail(e, "cudaGetDevice");
    return nullptr;
  }
  std::lock_guard<std::mutex> lk(g_mu);
  if ((int)g_ws.size() <= dev) g_ws.resize(dev + 1);
  auto& v = g_ws[dev];
  if (v.size() < kWsSlots) v.resize(kWsSlots);
  WsEntry& w = v[slot];
  if (w.bytes < bytes) {
    if (w.ptr) {
      cudaDeviceSynchronize();
      cudaFree(w.ptr);
      w.ptr = nullptr;
      w.bytes = 0;
    }
    size_t sz = (bytes + 255) & ~size_t(255);
    g_ws_allocs++;
    e = cudaMalloc(&w.ptr, sz);
    if (e != cudaSuccess) {
      cudaGetLastError();
      *status = cuda_fail(e, "cudaMalloc(workspace)");
      return nullptr;
    }
    e = cudaMemset(w.ptr, 0, sz);
    if (e != cudaSuccess) {
      *status = cuda_fail(e, "cudaMemset(workspace)");
      return nullptr;
    }
    w.bytes = sz;
  }
  return w.ptr;
}

void count_launch(int n) { g_launches += n; }

static WaitCtl g_wait_ctl;
WaitCtl wait_ctl() {
  std::lock_guard<std::mutex> lk(g_mu);
  return g_wait_ctl;
}
int set_wait_ctl(long long budget, int skip_cta) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_wait_ctl.budget = budget > 0 ? budget : kWaitBudget;
  g_wait_ctl.skip_cta = skip_cta >= 0 ? skip_cta : -1;
  return PERKS_OK;
}

int sync_words(SyncWords* out, cudaStream_t s) {
  int st = PERKS_OK;
  unsigned* w = static_cast<unsigned*>(workspace(kWsSync, 256, &st));
  if (!w) return st;
  PERKS_CUDA(cudaMemsetAsync(w, 0, 4 * sizeof(unsigned), s));
  out->bar = w;
  out->status = w + 2;
  return PERKS_OK;
}

int check_status(const SyncWords& w, cudaStream_t s) {
  unsigned h = 0;
  PERKS_CUDA(cudaMemcpyAsync(&h, w.status, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  PERKS_CUDA(cudaStreamSynchronize(s));
  if (h == 0) return PERKS_OK;
  if (h & kErrBreakdown) return fail(PERKS_ERR_BREAKDOWN, "CG breakdown: p.Ap <= 0 or non-finite (matrix not SPD?)");
  if (h & kErrNonFinite) return fail(PERKS_ERR_BREAKDOWN, "CG: non-finite residual");
  if (h & (kErrBarrierTimeout | kErrCopyTimeout))
    return fail(PERKS_ERR_TIMEOUT, "device-side wait exceeded its budget (status bits " + std::to_string(h) + ")");
  return fail(PERKS_ERR_CUDA, "device reported status " + std::to_string(h));
}

}  // namespace perks

extern "C" {

const char* perks_last_error(void) { return perks::g_last_error.c_str(); }

const char* perks_status_string(int status) {
  switch (status) {
    case PERKS_OK: return "ok";
    case PERKS_ERR_INVALID_ARG: return "invalid argument";
    case PERKS_ERR_UNSUPPORTED: return "unsupported configuration";
    case PERKS_ERR_NO_DEVICE: return "no usable CUDA device";
    case PERKS_ERR_CUDA: return "CUDA error";
    case PERKS_ERR_OOM: return "out of device memory";
    case PERKS_ERR_TIMEOUT: return "device-side wait timed out";
    case PERKS_ERR_LAUNCH: return "cooperative grid does not fit the device";
    case PERKS_ERR_BREAKDOWN: return "CG breakdown";
    case PERKS_ERR_NOT_CONVERGED: return "CG did not converge";
    default: return "unknown status";
  }
}

int perks_abi_version(void) { return PERKS_ABI_VERSION; }
long long perks_debug_workspace_allocs(void) {
  std::lock_guard<std::mutex> lk(perks::g_mu);
  return perks::g_ws_allocs;
}
int perks_debug_set_wait_fault(long long budget_cycles, int skip_cta) {
  return perks::set_wait_ctl(budget_cycles, skip_cta);
}
long long perks_launch_count(void) { return perks::g_launches; }
void perks_reset_launch_count(void) { perks::g_launches = 0; }

}  // extern "C"
