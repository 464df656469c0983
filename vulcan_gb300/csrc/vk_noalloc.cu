// Block-tridiagonal FP64 solve that allocates no memory.
//
// For callers that cannot call cudaMalloc: code running where a host-side
// allocation is not allowed or not wanted -- inside a framework that owns all
// device memory through its own pool, or a plugin handed pre-allocated
// buffers by its host -- and that still need the solver's scratch space.  The
// scratch (block inverses and the forward-sweep vector) lives in one
// file-scope __device__ array of fixed size, so nothing is allocated at call
// time; every GPU that loads the library holds that array until the process
// exits.  Each call waits for its stream to finish (it reads the status word
// back to report a singular or non-finite block).
//
// Solves, for one column of nz layers with ni species,
//     lower[j] o x[j-1] + D[j] x[j] + upper[j] o x[j+1] = b[j]
// (D dense ni x ni, lower/upper diagonal vectors) by block-Thomas with
// in-place Gauss-Jordan inversion of each Schur-complemented block, the same
// arithmetic as the FP64 Ros2 solver.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>
#include <string>

#include "vk_gj.cuh"
#include "vk_internal.cuh"

// Scratch capacity in doubles: nz*ni*ni (inverses) + nz*ni (sweep vector) + 1
// (status word) must fit.  2^21 doubles = 16 MiB, e.g. nz = 200 at ni = 100.
#define VK_NOALLOC_MAX_DOUBLES (1u << 21)

static __device__ __align__(256) double g_noalloc_scratch[VK_NOALLOC_MAX_DOUBLES];

namespace {

__global__ void __launch_bounds__(256)
k_block_solve_noalloc(int nz, int n, const double *__restrict__ D, const double *__restrict__ lo,
                      const double *__restrict__ up, const double *__restrict__ b,
                      double *__restrict__ x, double *__restrict__ scratch) {
    extern __shared__ double sm[];
    const int nn = n * n;
    double *G = scratch;                                  // [nz][n][n]
    double *z = scratch + (size_t)nz * nn;                // [nz][n]
    double *status = z + (size_t)nz * n;                  // one word, cleared here
    double *A = sm;
    double *colk = A + nn;
    double *rowk = colk + n;
    double *zp = rowk + n;
    double *bb = zp + n;
    int *perm = reinterpret_cast<int *>(bb + n);
    __shared__ int s_sing;
    const int tid = threadIdx.x, nth = blockDim.x, warp = tid >> 5, lane = tid & 31;
    const int nwarp = nth >> 5;
    if (tid == 0) s_sing = 0;
    for (int j = 0; j < nz; ++j) {
        const size_t l = (size_t)j;
        const double *lj = lo + l * n;
        const double *um = j > 0 ? up + (l - 1) * n : up;
        const double *Dj = D + l * nn;
        for (int e = tid; e < nn; e += nth) {
            int r = e / n, q = e - r * n;
            double v = Dj[e];
            if (j > 0) v -= lj[r] * A[e] * um[q];
            A[e] = v;
        }
        for (int t = tid; t < n; t += nth) bb[t] = b[l * n + t] - (j > 0 ? lj[t] * zp[t] : 0.0);
        __syncthreads();
        vk::gj_invert_f64(A, n, colk, rowk, perm, &s_sing);
        double *Gl = G + l * nn;
        for (int e = tid; e < nn; e += nth) Gl[e] = A[e];
        for (int r = warp; r < n; r += nwarp) {
            double s = 0.0;
            for (int q = lane; q < n; q += 32) s += A[r * n + q] * bb[q];
            for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if (lane == 0) rowk[r] = s;
        }
        __syncthreads();
        for (int t = tid; t < n; t += nth) {
            zp[t] = rowk[t];
            z[l * n + t] = rowk[t];
        }
        __syncthreads();
    }
    // back substitution: x_j = z_j - G_j (up_j o x_{j+1})
    double *xs = colk;
    for (int j = nz - 1; j >= 0; --j) {
        const size_t l = (size_t)j;
        if (j == nz - 1) {
            for (int t = tid; t < n; t += nth) rowk[t] = z[l * n + t];
        } else {
            const double *Gl = G + l * nn;
            for (int r = warp; r < n; r += nwarp) {
                double s = 0.0;
                for (int q = lane; q < n; q += 32) s += Gl[r * n + q] * xs[q];
                for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
                if (lane == 0) rowk[r] = z[l * n + r] - s;
            }
        }
        __syncthreads();
        for (int t = tid; t < n; t += nth) {
            x[l * n + t] = rowk[t];
            if (j > 0) xs[t] = up[(l - 1) * n + t] * rowk[t];
        }
        __syncthreads();
    }
    if (tid == 0) *status = (double)s_sing;
}

std::mutex g_setup_mu;
constexpr int kMaxDevices = 64;
double *g_scratch_dev[kMaxDevices] = {};   // device address of the array, per device
int noalloc_fail(int code, const std::string &msg) {
    vk::set_global_error(msg);        // read back with vk_last_error(NULL)
    return code;
}

// Once per device, with that device current: resolve the array's device
// address (host code must not use the symbol itself) and opt the kernel into
// the shared memory a 160-species block needs.
int noalloc_setup(int dev, double **out) {
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (!g_scratch_dev[dev]) {
        double *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress((void **)&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return noalloc_fail(VK_ECUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        size_t sm = (size_t)(VK_MAX_NI * VK_MAX_NI + 4 * VK_MAX_NI) * sizeof(double) + VK_MAX_NI * sizeof(int);
        e = cudaFuncSetAttribute(k_block_solve_noalloc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess)
            return noalloc_fail(VK_ECUDA, std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(e));
        g_scratch_dev[dev] = p;
    }
    *out = g_scratch_dev[dev];
    return VK_OK;
}

}  // namespace

extern "C" int vk_block_solve_noalloc(int nz, int ni, const double *D, const double *lower,
                                      const double *upper, const double *b, double *x,
                                      void *stream) {
    if (nz < 1 || ni < 1 || ni > VK_MAX_NI)
        return noalloc_fail(VK_EINVAL, "need nz >= 1 and 1 <= ni <= " + std::to_string(VK_MAX_NI));
    const unsigned long long need =
        (unsigned long long)nz * ni * ni + (unsigned long long)nz * ni + 1ull;
    if (need > VK_NOALLOC_MAX_DOUBLES)
        return noalloc_fail(VK_EINVAL, "nz*ni*ni + nz*ni + 1 = " + std::to_string(need) +
                                           " doubles exceeds the fixed scratch of " +
                                           std::to_string(VK_NOALLOC_MAX_DOUBLES) + " doubles (16 MiB)");
    if (!D || !lower || !upper || !b || !x) return noalloc_fail(VK_EINVAL, "NULL array");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return noalloc_fail(VK_ECUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return noalloc_fail(VK_EINVAL, "device ordinal out of range");
    double *scratch = nullptr;
    int rc = noalloc_setup(dev, &scratch);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    // an error left pending by earlier, unrelated work is reported as such
    // (and cleared) rather than blamed on this launch
    e = cudaGetLastError();
    if (e != cudaSuccess)
        return noalloc_fail(VK_ECUDA, std::string("CUDA error pending from earlier work (nothing launched): ") +
                                          cudaGetErrorString(e));
    size_t sm = (size_t)(ni * ni + 4 * ni) * sizeof(double) + (size_t)ni * sizeof(int);
    k_block_solve_noalloc<<<1, 256, sm, s>>>(nz, ni, D, lower, upper, b, x, scratch);
    e = cudaGetLastError();
    if (e != cudaSuccess) return noalloc_fail(VK_ECUDA, std::string("launch: ") + cudaGetErrorString(e));
    double status = 0.0;
    e = cudaMemcpyAsync(&status, scratch + (size_t)nz * ni * ni + (size_t)nz * ni, sizeof(double),
                        cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return noalloc_fail(VK_ECUDA, std::string("status read: ") + cudaGetErrorString(e));
    if (status == 1.0) return noalloc_fail(VK_ESINGULAR, "singular diagonal block");
    if (status == 2.0) return noalloc_fail(VK_ENAN, "non-finite pivot (NaN input)");
    return VK_OK;
}
