// gb_noalloc.cu -- the Gram product V^T W for callers that cannot allocate
// device memory.
//
// Some embedding applications own the whole GPU memory through their own pool
// or arena and may not call cudaMalloc / cudaFree (those calls can synchronise
// the device and would take memory the pool has already claimed). This entry
// point computes the same Gram block as GCGE_GPU_MultiVecInnerProd into memory
// the caller passes, with its partial sums in a fixed file-scope device array
// instead of the library's context scratch, and allocates nothing. It runs the
// FP64-pipe Gram kernels (k_gram_partial + k_gram_reduce, plain FP64 fused
// multiply-adds with a fixed-order second stage), not the tensor-core Gram: the
// tensor-core form needs per-call column-scale and digit buffers that would not
// fit a small fixed array.
//
// The array is GB_NOALLOC_DOUBLES doubles (8 MiB); every GPU that loads the
// library holds it until the process exits. All calls share it and it keeps the
// last call's contents: every call writes each partial it later reads, so
// nothing needs to start at zero. Calls that overlap on the GPU (different
// streams, or different host threads on one device) race on the array.
#include <cuda_runtime.h>

#include <atomic>
#include <mutex>

#include "gb_internal.h"

#define GB_NOALLOC_DOUBLES (1u << 20)
#define GB_NOALLOC_MAX_DEVICES 64

extern "C" int gb_gram_fixed_scratch(cudaStream_t stream, int num_sms, int n, int k1, int k2, const double *V,
                                     long ldv, const double *W, long ldw, double *a_dev, int lda, int sym,
                                     double *part, size_t part_cap);

static __device__ __align__(256) double g_noalloc_partials[GB_NOALLOC_DOUBLES];

// Per-device address of the array and SM count, set up on the first call on a
// device with that device current (host code must not pass the array's name:
// on the host it is only a stand-in symbol, not a device address). The set-up
// runs under a lock; the address is published with a release store after the SM
// count, and read with an acquire load, so a thread that sees the address also
// sees the count, whichever host thread made the first call.
static std::atomic<double *> s_part_addr[GB_NOALLOC_MAX_DEVICES];
static std::atomic<int> s_num_sms[GB_NOALLOC_MAX_DEVICES];
static std::mutex s_setup_lock;

static int setup_device(int dev, double **part, int *num_sms)
{
    double *p = s_part_addr[dev].load(std::memory_order_acquire);
    if (!p) {
        std::lock_guard<std::mutex> guard(s_setup_lock);
        p = s_part_addr[dev].load(std::memory_order_acquire);
        if (!p) {
            void *addr = nullptr;
            if (cudaGetSymbolAddress(&addr, g_noalloc_partials) != cudaSuccess || !addr) return GCGE_GPU_ERR_CUDA;
            int sms = 0;
            if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
                return GCGE_GPU_ERR_CUDA;
            s_num_sms[dev].store(sms, std::memory_order_relaxed);
            p = (double *)addr;
            s_part_addr[dev].store(p, std::memory_order_release);
        }
    }
    *part = p;
    *num_sms = s_num_sms[dev].load(std::memory_order_relaxed);
    return GCGE_GPU_OK;
}

extern "C" int GCGE_GPU_InnerProdNoAlloc(int n, int k1, int k2, const double *V, long ldv, const double *W, long ldw,
                                         double *a, int lda, int sym, void *stream)
{
    if (n <= 0 || k1 <= 0 || k2 <= 0 || !V || !W || !a || lda < k1 || ldv < k1 || ldw < k2 || (sym && k1 != k2))
        return GCGE_GPU_ERR_ARG;
    if ((size_t)k1 * k2 > GB_NOALLOC_DOUBLES / 4) return GCGE_GPU_ERR_ARG;   // at most 262,144 entries
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= GB_NOALLOC_MAX_DEVICES) return GCGE_GPU_ERR_CUDA;
    double *part = nullptr;
    int num_sms = 0;
    int st = setup_device(dev, &part, &num_sms);
    if (st) return st;
    return gb_gram_fixed_scratch((cudaStream_t)stream, num_sms, n, k1, k2, V, ldv, W, ldw, a, lda, sym, part,
                                 GB_NOALLOC_DOUBLES);
}
