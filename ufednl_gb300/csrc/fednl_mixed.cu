// fednl_mixed.cu -- host side of the tensor-core (tcgen05) path: tensor maps, the feature-major
// layout of dense FP32 client data, and the operator-level weighted Gram entry point.
//
// Layout: client c's features are stored feature-major, X[c][i][s] (d rows, L columns, L = the
// largest n_i rounded up to 32, zero beyond n_c), so that a TMA box of 32 samples x 128 features is
// one 128-byte-swizzled K-major UMMA operand slab.  The per-sample weights D_s live in W[c][s]
// (zero beyond n_c, so the padding contributes nothing).

#include "fednl_gpu.h"
#include "fednl_tc.cuh"

#include <cudaTypedefs.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <string>
#include <vector>

extern "C" const char* fednl_gpu_last_error(void);
int fednl_set_error(int code, const char* msg);   // fednl_gpu.cu

namespace {

int fail_m(int code, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    return fednl_set_error(code, buf);
}

#define CKM(call)                                                                                  \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess)                                                                     \
            return fail_m(FEDNL_ECUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
    } while (0)

PFN_cuTensorMapEncodeTiled_v12000 encode_fn()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        cudaDriverEntryPointQueryResult q;
        void* p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    }
    return fn;
}

// [nc][d][L] FP32, box = 32 samples x 128 features x 1 client, 128-byte swizzle
int make_feature_map(CUtensorMap* map, const float* X, int L, int d, int nc)
{
    auto fn = encode_fn();
    if (!fn) return fail_m(FEDNL_ECUDA, "cuTensorMapEncodeTiled is not available");
    cuuint64_t dims[3] = {(cuuint64_t)L, (cuuint64_t)d, (cuuint64_t)nc};
    cuuint64_t strides[2] = {(cuuint64_t)L * 4, (cuuint64_t)L * d * 4};
    cuuint32_t box[3] = {(cuuint32_t)fednl_tc::kBK, (cuuint32_t)fednl_tc::kBM, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, (void*)X, dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail_m(FEDNL_ECUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return FEDNL_OK;
}

// sample-major [sum n][d] (clients in order) -> feature-major [nc][d][L], zero padding
__global__ void k_to_feature_major(const float* __restrict__ A, const int* __restrict__ soff, int d, int L, int nc,
                                   float* __restrict__ X)
{
    __shared__ float tile[32][33];
    const int c = blockIdx.z;
    const int s0 = blockIdx.x * 32, i0 = blockIdx.y * 32;
    const int n = soff[c + 1] - soff[c];
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int s = s0 + r, i = i0 + threadIdx.x;
        tile[r][threadIdx.x] = (s < n && i < d) ? A[(size_t)(soff[c] + s) * d + i] : 0.0f;
    }
    __syncthreads();
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int i = i0 + r, s = s0 + threadIdx.x;
        if (i < d && s < L) X[((size_t)c * d + i) * L + s] = tile[threadIdx.x][r];
    }
}

__global__ void k_pad_weights(const float* __restrict__ w, const int* __restrict__ soff, int L, int nc,
                              float* __restrict__ W)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x, c = blockIdx.y;
    const int n = soff[c + 1] - soff[c];
    if (s < L) W[(size_t)c * L + s] = s < n ? w[soff[c] + s] : 0.0f;
}

}  // namespace

extern "C" int fednl_gpu_weighted_gram_tf32(const float* features, const float* weights, const int32_t* n_samples,
                                            int32_t n_clients, int32_t d, float lambda, float* out)
{
    if (!features || !weights || !n_samples || !out || n_clients < 1 || d < 128 || d % 128)
        return fail_m(FEDNL_EINVAL, "bad argument (d must be a positive multiple of 128)");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail_m(FEDNL_ENODEV, "no CUDA device available");
    std::vector<int> soff(n_clients + 1, 0);
    int maxn = 0;
    for (int c = 0; c < n_clients; ++c) {
        if (n_samples[c] < 1) return fail_m(FEDNL_EINVAL, "client %d has no samples", c);
        soff[c + 1] = soff[c] + n_samples[c];
        maxn = std::max(maxn, n_samples[c]);
    }
    const int S = soff[n_clients];
    const int L = (maxn + 31) / 32 * 32;
    float *dA = nullptr, *dw = nullptr, *dX = nullptr, *dW = nullptr, *dout = nullptr;
    int *dsoff = nullptr, *dns = nullptr, *derr = nullptr;
    auto cleanup = [&]() {
        cudaFree(dA);
        cudaFree(dw);
        cudaFree(dX);
        cudaFree(dW);
        cudaFree(dout);
        cudaFree(dsoff);
        cudaFree(dns);
        cudaFree(derr);
    };
    const size_t outN = (size_t)n_clients * d * d;
    if (cudaMalloc(&dA, (size_t)S * d * 4) != cudaSuccess || cudaMalloc(&dw, (size_t)S * 4) != cudaSuccess ||
        cudaMalloc(&dX, (size_t)n_clients * d * L * 4) != cudaSuccess ||
        cudaMalloc(&dW, (size_t)n_clients * L * 4) != cudaSuccess || cudaMalloc(&dout, outN * 4) != cudaSuccess ||
        cudaMalloc(&dsoff, (n_clients + 1) * 4) != cudaSuccess || cudaMalloc(&dns, n_clients * 4) != cudaSuccess ||
        cudaMalloc(&derr, 4) != cudaSuccess) {
        cleanup();
        return fail_m(FEDNL_ENOMEM, "device allocation failed");
    }
    int rc = FEDNL_OK;
    do {
        if (cudaMemcpy(dA, features, (size_t)S * d * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(dw, weights, (size_t)S * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(dsoff, soff.data(), (n_clients + 1) * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(dns, n_samples, n_clients * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemset(dout, 0, outN * 4) != cudaSuccess || cudaMemset(derr, 0, 4) != cudaSuccess) {
            rc = fail_m(FEDNL_ECUDA, "copies failed");
            break;
        }
        k_to_feature_major<<<dim3(L / 32, (d + 31) / 32, n_clients), dim3(32, 8)>>>(dA, dsoff, d, L, n_clients, dX);
        k_pad_weights<<<dim3((L + 255) / 256, n_clients), 256>>>(dw, dsoff, L, n_clients, dW);
        CUtensorMap map;
        rc = make_feature_map(&map, dX, L, d, n_clients);
        if (rc) break;
        fednl_tc::GramJob J;
        J.d = d;
        J.nc = n_clients;
        J.L = L;
        J.nbk = d / fednl_tc::kBM;
        J.tiles = J.nbk * (J.nbk + 1) / 2;
        J.ns = dns;
        J.act = nullptr;
        J.w = dW;
        J.err = derr;
        fednl_tc::EpiStore epi{dout, d, lambda};
        const size_t smem = fednl_tc::smem_bytes();
        if (cudaFuncSetAttribute(fednl_tc::k_gram_tf32<fednl_tc::EpiStore>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem) != cudaSuccess) {
            rc = fail_m(FEDNL_ECUDA, "shared-memory attribute refused");
            break;
        }
        fednl_tc::k_gram_tf32<fednl_tc::EpiStore><<<n_clients * J.tiles, fednl_tc::kThreads, smem>>>(map, J, epi);
        cudaError_t e = cudaDeviceSynchronize();
        if (e != cudaSuccess) {
            rc = fail_m(FEDNL_ECUDA, "Gram kernel failed: %s", cudaGetErrorString(e));
            break;
        }
        int err = 0;
        cudaMemcpy(&err, derr, 4, cudaMemcpyDeviceToHost);
        if (err) {
            rc = fail_m(FEDNL_ETIMEOUT, "a bounded wait of the Gram kernel ran out");
            break;
        }
        if (cudaMemcpy(out, dout, outN * 4, cudaMemcpyDeviceToHost) != cudaSuccess) rc = fail_m(FEDNL_ECUDA, "readback failed");
    } while (0);
    cleanup();
    return rc;
}
