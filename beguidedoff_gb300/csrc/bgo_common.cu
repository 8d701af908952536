// Error state, version, device count and pinned host buffers of the C ABI.
#include <string.h>

#include <mutex>
#include <string>
#include <vector>

#include "bgo_internal.cuh"

namespace bgo {

namespace {
constexpr int kPoolDevices = 64;
std::mutex g_pool_mu;
cudaMemPool_t g_pool[kPoolDevices];
cudaStream_t g_free_stream[kPoolDevices];

// The device's pool (created on first use, keeping freed memory for reuse)
// and the stream frees are ordered on.
cudaError_t device_pool(int device, cudaMemPool_t *pool, cudaStream_t *free_stream) {
    if (device < 0 || device >= kPoolDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_pool_mu);
    if (!g_pool[device]) {
        cudaMemPoolProps props{};
        props.allocType = cudaMemAllocationTypePinned;
        props.handleTypes = cudaMemHandleTypeNone;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = device;
        cudaMemPool_t p = nullptr;
        cudaError_t e = cudaMemPoolCreate(&p, &props);
        if (e != cudaSuccess) return e;
        uint64_t keep = ~0ull;
        e = cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep);
        cudaStream_t fs = nullptr;
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&fs, cudaStreamNonBlocking);
        // map 64 MB up front: growing the pool later waits for the device
        void *warm = nullptr;
        if (e == cudaSuccess) e = cudaMallocFromPoolAsync(&warm, 64u << 20, p, fs);
        if (e == cudaSuccess) e = cudaFreeAsync(warm, fs);
        if (e == cudaSuccess) e = cudaStreamSynchronize(fs);
        if (e != cudaSuccess) {
            if (fs) cudaStreamDestroy(fs);
            cudaMemPoolDestroy(p);
            return e;
        }
        g_pool[device] = p;
        g_free_stream[device] = fs;
    }
    *pool = g_pool[device];
    *free_stream = g_free_stream[device];
    return cudaSuccess;
}
}  // namespace

// Allocations and frees are both ordered on the pool's own stream, so a freed
// block is always reusable by the next allocation (a block freed on another
// stream may not be, and the pool then maps new memory, which waits for the
// device).  The stream holds only these operations: synchronising it after an
// allocation waits for nothing else.
cudaError_t pool_alloc(int device, void **p, size_t bytes) {
    cudaMemPool_t pool = nullptr;
    cudaStream_t fs = nullptr;
    cudaError_t e = device_pool(device, &pool, &fs);
    if (e != cudaSuccess) return e;
    e = cudaMallocFromPoolAsync(p, bytes ? bytes : 1, pool, fs);
    if (e == cudaSuccess) e = cudaStreamSynchronize(fs);
    return e;
}

// Events that mark a plan's last use are recycled: creating and destroying an
// event can wait for the device while other streams run.
namespace {
std::mutex g_event_mu;
std::vector<cudaEvent_t> g_events[kPoolDevices];
}  // namespace

cudaError_t event_take(int device, cudaEvent_t *ev) {
    if (device < 0 || device >= kPoolDevices) return cudaErrorInvalidDevice;
    {
        std::lock_guard<std::mutex> lock(g_event_mu);
        if (!g_events[device].empty()) {
            *ev = g_events[device].back();
            g_events[device].pop_back();
            return cudaSuccess;
        }
    }
    return cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
}

void event_give(int device, cudaEvent_t ev) {
    if (!ev) return;
    if (device < 0 || device >= kPoolDevices) {
        cudaEventDestroy(ev);
        return;
    }
    std::lock_guard<std::mutex> lock(g_event_mu);
    g_events[device].push_back(ev);
}

cudaError_t pool_free(int device, void *p) {
    if (!p) return cudaSuccess;
    cudaMemPool_t pool = nullptr;
    cudaStream_t fs = nullptr;
    cudaError_t e = device_pool(device, &pool, &fs);
    if (e != cudaSuccess) return e;
    return cudaFreeAsync(p, fs);
}

cudaError_t pool_free_after(int device, void *p, cudaStream_t stream) {
    if (!p) return cudaSuccess;
    cudaMemPool_t pool = nullptr;
    cudaStream_t fs = nullptr;
    cudaError_t e = device_pool(device, &pool, &fs);
    if (e != cudaSuccess) return e;
    cudaEvent_t ev = nullptr;
    e = event_take(device, &ev);
    if (e == cudaSuccess) e = cudaEventRecord(ev, stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(fs, ev, 0);
    if (e == cudaSuccess) e = cudaFreeAsync(p, fs);
    // the event may be re-recorded once the free stream has taken its wait
    event_give(device, ev);
    return e;
}

static thread_local std::string g_last_error;

void set_error(const std::string &msg) { g_last_error = msg; }

int cuda_fail(cudaError_t e, const char *what) {
    set_error(std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")");
    return e == cudaErrorMemoryAllocation ? BGO_ERR_OOM : BGO_ERR_CUDA;
}

}  // namespace bgo

extern "C" int bgo_version(void) { return 100; }

extern "C" int bgo_last_error(char *buf, size_t len) {
    if (!buf || len == 0) return BGO_ERR_ARG;
    size_t n = bgo::g_last_error.size();
    if (n >= len) n = len - 1;
    memcpy(buf, bgo::g_last_error.data(), n);
    buf[n] = '\0';
    return BGO_OK;
}

extern "C" int bgo_device_count(int *n) {
    if (!n) return BGO_ERR_ARG;
    int c = 0;
    cudaError_t e = cudaGetDeviceCount(&c);
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) {
        cudaGetLastError();
        *n = 0;
        return BGO_OK;
    }
    BGO_CUDA(e);
    *n = c;
    return BGO_OK;
}

extern "C" int bgo_host_alloc(void **ptr, size_t bytes) {
    if (!ptr) return BGO_ERR_ARG;
    BGO_CUDA(cudaHostAlloc(ptr, bytes ? bytes : 1, cudaHostAllocDefault));
    return BGO_OK;
}

extern "C" int bgo_host_free(void *ptr) {
    if (ptr) BGO_CUDA(cudaFreeHost(ptr));
    return BGO_OK;
}

extern "C" int bgo_stream_create(int device, void **stream) {
    if (!stream) return BGO_ERR_ARG;
    *stream = nullptr;
    BGO_CUDA(cudaSetDevice(device));
    cudaStream_t s = nullptr;
    BGO_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    *stream = (void *)s;
    return BGO_OK;
}

extern "C" int bgo_stream_destroy(void *stream) {
    if (!stream) return BGO_OK;
    BGO_CUDA(cudaStreamDestroy((cudaStream_t)stream));
    return BGO_OK;
}
