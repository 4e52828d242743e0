// LOD scoring without device allocation (sl_lod_score_device_graphs_noalloc).
//
// Some callers cannot call cudaMalloc where they score: a host that reserves
// the device's memory up front through its own allocator, or a latency-bound
// loop where cudaMalloc/cudaFree, which can synchronise the device, would
// stall other streams.  This entry point therefore keeps its scratch -- the
// log-likelihood ratio of every (graph, interval, position) before the
// in-order log-sum -- in the file-scope array below, sized
// SL_NOALLOC_SCRATCH_BYTES.  The array is held by every GPU that loads the
// library until the process exits.  Host code must not hand the array's name
// to a kernel (on the host it is only a stand-in for the device symbol): the
// device address is looked up with cudaGetSymbolAddress once per device, on
// the first call made with that device current; the caller's current device
// is restored before the call returns.  Every call overwrites the whole
// region it uses before reading it, so nothing needs clearing; calls that
// overlap on the GPU share the array and race.  The scores come from the
// kernel the context scores with (sl_lod_score_graphs).

#include <cuda_runtime.h>
#include <float.h>
#include <mutex>

#include "../../include/swiftlink_gb300.h"
#include "sl_internal.h"

namespace sl {
int ctx_view(sl_ctx* ctx, CtxView* v);
void ctx_fail(sl_ctx* ctx, int code, const char* msg);
cudaError_t ctx_launch_lod(sl_ctx* ctx, const uint32_t* graphs, int G, double* vals);
cudaError_t launch_lod_merge(const double* vals, int G, int64_t npos, double* acc, uint8_t* init, cudaStream_t s);
}  // namespace sl

namespace {
const size_t kScratchDoubles = SL_NOALLOC_SCRATCH_BYTES / sizeof(double);
static __device__ __align__(256) double g_lod_scratch[SL_NOALLOC_SCRATCH_BYTES / sizeof(double)];

const int kMaxDevices = 64;
std::mutex g_lock;
double* g_scratch_addr[kMaxDevices] = {nullptr};

// Device address of the scratch array on `device`, looked up once per device
// (the caller has made `device` current).
int scratch_for(int device, double** out) {
    if (device < 0 || device >= kMaxDevices) return SL_EINVAL;
    std::lock_guard<std::mutex> guard(g_lock);
    if (!g_scratch_addr[device]) {
        void* ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_lod_scratch);
        if (e != cudaSuccess || !ptr) return SL_ECUDA;
        g_scratch_addr[device] = (double*)ptr;
    }
    *out = g_scratch_addr[device];
    return SL_OK;
}

// Makes the context's device current for the call and gives the caller's
// thread its own current device back on return.
struct DeviceGuard {
    int prev = -1;
    bool ok = false;
    explicit DeviceGuard(int device) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        ok = cudaSetDevice(device) == cudaSuccess;
    }
    ~DeviceGuard() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};
}  // namespace

extern "C" int sl_lod_score_device_graphs_noalloc(sl_ctx* ctx, int32_t n_graphs, const uint32_t* d_graphs,
                                                  double* d_logsum) {
    using namespace sl;
    CtxView v;
    if (ctx_view(ctx, &v) != SL_OK) return SL_EINVAL;
    if (n_graphs < 1 || !d_graphs || !d_logsum) {
        ctx_fail(ctx, SL_EINVAL, "noalloc LOD scoring: need n_graphs >= 1 and device buffers");
        return SL_EINVAL;
    }
    const int64_t npos = (int64_t)(v.P.M - 1) * v.P.n_lod;
    if ((int64_t)n_graphs * npos > (int64_t)kScratchDoubles) {
        ctx_fail(ctx, SL_EINVAL,
                 "noalloc LOD scoring: n_graphs * positions exceeds the 8 MiB scratch array "
                 "(1048576 values); score fewer graphs per call");
        return SL_EINVAL;
    }
    DeviceGuard dev(v.device);
    if (!dev.ok) {
        ctx_fail(ctx, SL_ECUDA, "noalloc LOD scoring: cudaSetDevice failed");
        return SL_ECUDA;
    }
    double* scratch = nullptr;
    int rc = scratch_for(v.device, &scratch);
    if (rc != SL_OK) {
        ctx_fail(ctx, rc, "noalloc LOD scoring: cudaGetSymbolAddress of the scratch array failed");
        return rc;
    }
    cudaStream_t s = (cudaStream_t)v.stream;
    cudaError_t e = ctx_launch_lod(ctx, d_graphs, n_graphs, scratch);
    if (e == cudaSuccess) e = launch_lod_merge(scratch, n_graphs, npos, d_logsum, nullptr, s);
    if (e != cudaSuccess) {
        ctx_fail(ctx, SL_ECUDA, cudaGetErrorString(e));
        return SL_ECUDA;
    }
    return SL_OK;
}
