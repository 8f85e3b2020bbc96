// Host runtime: per-device contexts, error strings, basis classification and
// the exact squared-distance limits.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <cstdlib>
#include <map>

#include "frmc_runtime.h"

namespace frmc {

static thread_local char g_err[512] = "";

int set_error(int code, const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}

const char *last_error() { return g_err; }

int cuda_fail(cudaError_t e, const char *what)
{
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        return set_error(FRMC_E_NOMEM, "%s: %s", what, cudaGetErrorString(e));
    }
    return set_error(FRMC_E_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

int DevBuf::ensure(size_t bytes)
{
    if (bytes <= cap && p)
        return FRMC_OK;
    size_t want = bytes < 256 ? 256 : bytes;
    want = want + want / 4;  // headroom: grow geometrically
    if (p) {
        cudaFree(p);
        p = nullptr;
        cap = 0;
    }
    cudaError_t e = cudaMalloc(&p, want);
    if (e != cudaSuccess) {
        p = nullptr;
        return cuda_fail(e, "cudaMalloc");
    }
    cap = want;
    return FRMC_OK;
}

static std::mutex g_ctx_mu;
static std::map<int, Context *> g_ctx;

int get_context(Context **out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_error(FRMC_E_NODEV, "no CUDA device: %s", cudaGetErrorString(e));
    }
    std::lock_guard<std::mutex> lk(g_ctx_mu);
    auto it = g_ctx.find(dev);
    if (it != g_ctx.end()) {
        *out = it->second;
        return FRMC_OK;
    }
    Context *c = new Context();
    c->device = dev;
    FRMC_CUDA(cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, dev));
    FRMC_CUDA(cudaDeviceGetAttribute(&c->max_smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess) {
            cudaGetLastError();
            v = 0;
        }
        const char *env = std::getenv("FRMC_HOST_DIRECT");
        c->pageable = (v == 1 && !(env && env[0] == '0')) ? 1 : 0;
    }
    FRMC_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    g_ctx[dev] = c;
    *out = c;
    return FRMC_OK;
}

int basis_mode(const float *B, int isPBC)
{
    if (!isPBC)
        return BM_IBC;
    // B[r*3 + c]: rows are the box vectors.
    const bool z01 = B[1] == 0.0f, z02 = B[2] == 0.0f, z10 = B[3] == 0.0f, z12 = B[5] == 0.0f;
    const bool z20 = B[6] == 0.0f, z21 = B[7] == 0.0f;
    if (z01 && z02 && z10 && z12 && z20 && z21)
        return BM_DIAG;
    if (z01 && z02 && z12 && z20 && z21)
        return BM_XYTRI;
    if (z01 && z02 && z12)
        return BM_LOWER;
    return BM_GENERAL;
}

Basis make_basis(const float *B)
{
    Basis b;
    for (int k = 0; k < 9; ++k) b.b[k] = B ? B[k] : (k % 4 == 0 ? 1.0f : 0.0f);
    return b;
}

static inline float bits_to_f(uint32_t u)
{
    float f;
    memcpy(&f, &u, 4);
    return f;
}

// Smallest non-negative float s with sqrtf(s) >= limit (limit > 0, finite):
// sqrtf is correctly rounded, hence monotone, so a bisection over the bit
// patterns of non-negative floats (which are ordered like the values) finds it.
static float sqrt_threshold(float limit)
{
    uint32_t lo = 0u, hi = 0x7f800000u;  // +inf: sqrtf(inf) = inf >= limit
    while (lo < hi) {
        uint32_t mid = lo + (hi - lo) / 2u;
        if (std::sqrt(bits_to_f(mid)) >= limit)
            hi = mid;
        else
            lo = mid + 1u;
    }
    return bits_to_f(lo);
}

void sq_limits(float minD, float maxD, float *s_lo, float *s_hi)
{
    // d >= minD for every d >= 0 when minD <= 0 (or is NaN: d < NaN is false).
    if (!(minD > 0.0f))
        *s_lo = 0.0f;
    else if (std::isinf(minD))
        *s_lo = INFINITY;
    else
        *s_lo = sqrt_threshold(minD);
    // accept d < maxD: none when maxD <= 0; all finite when maxD is +inf/NaN.
    if (std::isnan(maxD) || (std::isinf(maxD) && maxD > 0))
        *s_hi = INFINITY;
    else if (!(maxD > 0.0f))
        *s_hi = 0.0f;
    else
        *s_hi = sqrt_threshold(maxD);
}

}  // namespace frmc
