// runtime.cu -- status reporting and the device error word of libqmcgb.
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <map>
#include <mutex>
#include <utility>

#include "common.cuh"

namespace qmcgb {

static thread_local char g_msg[512] = "";

void set_error(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_msg, sizeof(g_msg), fmt, ap);
    va_end(ap);
}

int cuda_status(cudaError_t e, const char *what)
{
    if (e == cudaSuccess) return QMC_OK;
    set_error("%s: %s", what, cudaGetErrorString(e));
    return QMC_ERR_CUDA;
}

int launch_status(const char *what) { return cuda_status(cudaGetLastError(), what); }

int raise_smem_limit(const void *func, size_t bytes, const char *what)
{
    if (bytes <= 48 * 1024) return QMC_OK;
    static std::mutex mu;
    static std::map<std::pair<int, const void *>, size_t> high;
    int dev = 0;
    if (int rc = cuda_status(cudaGetDevice(&dev), what)) return rc;
    std::lock_guard<std::mutex> lock(mu);
    size_t &cur = high[{dev, func}];
    if (bytes <= cur) return QMC_OK;
    if (int rc = cuda_status(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes), what))
        return rc;
    cur = bytes;
    return QMC_OK;
}

// One word per loaded library and device; kernels OR error codes into it.
__device__ unsigned int g_device_error;

unsigned int *device_error_ptr()
{
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_device_error) != cudaSuccess) return nullptr;
    return (unsigned int *)p;
}

int device_error_reset(cudaStream_t s)
{
    unsigned int *p = device_error_ptr();
    if (!p) return cuda_status(cudaGetLastError(), "locating the device error word");
    return cuda_status(cudaMemsetAsync(p, 0, sizeof(unsigned int), s), "clearing the device error word");
}

int sm_count()
{
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 152;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 152;
    return n > 0 ? n : 152;
}

}  // namespace qmcgb

extern "C" {

const char *qmc_last_error(void) { return qmcgb::g_msg; }

int qmc_version(void) { return 10000; }

int qmc_device_error_reset(qmc_stream_t s) { return qmcgb::device_error_reset(QMC_STREAM(s)); }

int qmc_device_error_check(qmc_stream_t s)
{
    cudaStream_t st = QMC_STREAM(s);
    unsigned int *p = qmcgb::device_error_ptr();
    if (!p) return qmcgb::cuda_status(cudaGetLastError(), "locating the device error word");
    unsigned int h = 0;
    int rc = qmcgb::cuda_status(cudaMemcpyAsync(&h, p, sizeof(h), cudaMemcpyDeviceToHost, st),
                                "reading the device error word");
    if (rc) return rc;
    rc = qmcgb::cuda_status(cudaStreamSynchronize(st), "synchronising the stream");
    if (rc) return rc;
    if (h) {
        qmcgb::device_error_reset(st);
        qmcgb::set_error("device error word %u:%s%s%s%s", h, (h & 1u) ? " a table index outside its array;" : "",
                         (h & 2u) ? " a base below 2;" : "", (h & 4u) ? " a tensor-core completion wait ran out;" : "",
                         (h & 8u) ? " a fused generalized-net matrix entry at or above 2^32;" : "");
        return QMC_ERR_DEVICE;
    }
    return QMC_OK;
}

// Device-side address of host memory a kernel may write directly: memory
// pinned with cudaHostAlloc/cudaHostRegister is mapped into the device's
// address space under unified addressing.  Pageable memory is reported as not
// usable (returns QMC_ERR_ARG) even where the platform could reach it.
int qmc_host_pointer_for_device(const void *host, void **dev)
{
    if (!host || !dev) {
        qmcgb::set_error("null pointer");
        return QMC_ERR_ARG;
    }
    cudaPointerAttributes attr;
    cudaError_t e = cudaPointerGetAttributes(&attr, host);
    if (e != cudaSuccess) {
        cudaGetLastError();
        qmcgb::set_error("cudaPointerGetAttributes: %s", cudaGetErrorString(e));
        return QMC_ERR_ARG;
    }
    if (attr.type != cudaMemoryTypeHost || attr.devicePointer == nullptr) {
        qmcgb::set_error("host memory is not pinned and mapped");
        return QMC_ERR_ARG;
    }
    *dev = attr.devicePointer;
    return QMC_OK;
}

// Attributes of the current device that decide how host buffers are
// reached: pageable-memory access, whether it goes through the host page
// tables, and the SM count.
int qmc_device_attributes(int *pageable_access, int *uses_host_page_tables, int *sms)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return qmcgb::cuda_status(e, "cudaGetDevice");
    int a = 0, b = 0, c = 0;
    cudaDeviceGetAttribute(&a, cudaDevAttrPageableMemoryAccess, dev);
    cudaDeviceGetAttribute(&b, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev);
    cudaDeviceGetAttribute(&c, cudaDevAttrMultiProcessorCount, dev);
    if (pageable_access) *pageable_access = a;
    if (uses_host_page_tables) *uses_host_page_tables = b;
    if (sms) *sms = c;
    return qmcgb::cuda_status(cudaGetLastError(), "cudaDeviceGetAttribute");
}

}  // extern "C"
