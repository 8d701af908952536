// Error state, version, device count and pinned host buffers of the C ABI.
#include <string.h>

#include <string>

#include "bgo_internal.cuh"

namespace bgo {

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
