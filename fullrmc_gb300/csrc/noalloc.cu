// All-pairs histogram that allocates no device memory.
//
// Some callers cannot let a library call cudaMalloc: a host framework that
// hands out all device memory from its own pool (a stray cudaMalloc would
// fragment or overrun the pool's budget), or a stepping loop that must not
// stall, since cudaMalloc and cudaFree can synchronise the device.  For them,
// frmc_dev_full_pairs_histograms_noalloc computes the same histograms as
// full_pairs_histograms_coords into float32 buffers the caller owns, and keeps
// its uint32 counts and its status word in one fixed array of device memory
// reserved when the library is loaded (below).  Every GPU that loads the
// library holds that array until the process exits.
#include <climits>
#include <cstdio>
#include <mutex>

#include "frmc_gpu.h"
#include "frmc_runtime.h"

namespace frmc {

// Counts for intra plus inter: 2 * ne * ne * hs must not exceed this
// (4 MiB of uint32; e.g. ne = 4 and hs = 32768, or ne = 8 and hs = 8192).
constexpr long long kNoAllocMaxCounts = 1ll << 20;
constexpr long long kNoAllocWords = kNoAllocMaxCounts + 64;  // + status word and padding

// The fixed scratch array.  In host code this name is only a stand-in for the
// symbol, not a device address: host code passes the address obtained from
// cudaGetSymbolAddress to the kernels.
static __device__ __align__(256) unsigned int g_noalloc_scratch[kNoAllocWords];

struct NoAllocDevice {
    unsigned *scratch = nullptr;  // device address of g_noalloc_scratch on this device
    int sms = 0;
    int max_smem_optin = 0;
    bool ready = false;
};

constexpr int kMaxDevices = 64;
static std::mutex g_noalloc_mu;
static NoAllocDevice g_noalloc_dev[kMaxDevices];

// Once per device, with that device current: resolve the array's device
// address and read the launch limits.  Done by the first call on a device.
static int noalloc_setup(int dev, NoAllocDevice **out)
{
    if (dev < 0 || dev >= kMaxDevices)
        return set_error(FRMC_E_ARG, "device %d out of range for the no-allocation entry point", dev);
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    NoAllocDevice &d = g_noalloc_dev[dev];
    if (!d.ready) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess)
            return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        FRMC_CUDA(cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, dev));
        FRMC_CUDA(cudaDeviceGetAttribute(&d.max_smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
        d.scratch = static_cast<unsigned *>(p);
        d.ready = true;
    }
    *out = &d;
    return FRMC_OK;
}

}  // namespace frmc

using namespace frmc;

extern "C" {

int frmc_dev_full_pairs_histograms_noalloc(const void *atoms4, const int32_t *moleculeIndex, int64_t n,
                                           const float *basis_host, int isPBC, int32_t ne, float minDistance,
                                           float maxDistance, float bin, int32_t hs, float *hintra, float *hinter,
                                           void *stream)
{
    // the same atom limit as frmc_dev_full_hist_counts
    if (n < 0 || n > (int64_t)(INT_MAX / 4))
        return set_error(FRMC_E_ARG, "no-allocation histogram: %lld atoms out of range", (long long)n);
    if (ne < 0 || hs < 0)
        return set_error(FRMC_E_ARG, "no-allocation histogram: negative histogram shape (%d, %d)", ne, hs);
    const long long total = (long long)ne * ne * hs;
    if (2 * total > kNoAllocMaxCounts)
        return set_error(FRMC_E_ARG,
                         "no-allocation histogram: 2*ne*ne*hs = %lld counts exceed its fixed scratch of %lld counts",
                         2 * total, kNoAllocMaxCounts);
    if (total == 0)
        return FRMC_OK;
    if (n >= 2 && (((uintptr_t)atoms4 & 15u) || ((uintptr_t)moleculeIndex & 15u)))
        return set_error(FRMC_E_ARG, "no-allocation histogram: atoms4 and moleculeIndex must be 16-byte aligned");
    int dev = 0;
    FRMC_CUDA(cudaGetDevice(&dev));
    NoAllocDevice *d = nullptr;
    FRMC_TRY(noalloc_setup(dev, &d));
    cudaStream_t st = (cudaStream_t)stream;
    unsigned *counts = d->scratch;
    uint32_t *status = d->scratch + kNoAllocMaxCounts;
    // The array keeps the previous call's contents: clear what must start at zero.
    FRMC_CUDA(cudaMemsetAsync(counts, 0, sizeof(unsigned) * 2 * total, st));
    FRMC_CUDA(cudaMemsetAsync(status, 0, sizeof(uint32_t), st));
    if (n >= 2) {
        const float *B = isPBC ? basis_host : nullptr;
        static const float kId[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
        const float *Bh = B ? B : kId;
        FullTune tn = current_tune();
        FRMC_TRY(launch_full_hist_on(d->sms, d->max_smem_optin, (const float4 *)atoms4, moleculeIndex, (int)n,
                                     basis_mode(Bh, isPBC), make_basis(Bh), minDistance, maxDistance, bin, ne, hs,
                                     counts, counts + total, status,
                                     accept_fraction(Bh, isPBC, minDistance, maxDistance), &tn, st));
    }
    FRMC_TRY(launch_counts_to_f32(counts, nullptr, hintra, total, st));
    FRMC_TRY(launch_counts_to_f32(counts + total, nullptr, hinter, total, st));
    uint32_t host_status = 0;
    FRMC_CUDA(cudaMemcpyAsync(&host_status, status, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    FRMC_CUDA(cudaStreamSynchronize(st));
    if (host_status)
        return set_error(FRMC_E_TIMEOUT, "no-allocation histogram: a device wait gave up (status 0x%x)", host_status);
    return FRMC_OK;
}

}  // extern "C"
