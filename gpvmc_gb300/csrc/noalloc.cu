// Allocation-free Slater-matrix inversion: gv_slater_invert_noalloc.
//
// Some callers cannot let a library allocate device memory: applications
// that size their HBM once at start-up and hand out only pre-allocated
// buffers afterwards (a fixed arena shared with other solvers), and
// latency-critical loops where a cudaMalloc/cudaFree, with its implicit
// device synchronisation, is not acceptable.  This entry point serves them:
// the caller passes device pointers for the input and the outputs, and the
// one working buffer the inversion needs -- an FP64 complex N x N matrix --
// is a file-scope static __device__ array of fixed size.
//
// Limits and sharing rules:
//  * N <= GV_NOALLOC_MAX_N (128, i.e. lattices up to L = 16 at half filling);
//    the scratch is 128 * 128 * 16 B = 256 KiB, and every GPU that loads this
//    library holds it until the process exits.
//  * Every call uses the same array; it keeps the previous call's contents,
//    and each call overwrites the N x N block it uses before reading it.
//    Calls whose kernels overlap on a GPU (different streams, different host
//    threads) race on the array: serialise them.
//  * The device address of the array is looked up once per device, with
//    that device current, on the first call made there; make that first call
//    before any stream capture.  The address stays valid for the life of the
//    device's primary context: a caller that runs cudaDeviceReset must not
//    call this entry point on that device afterwards.
//  * A matrix that fails linalg::DetInv's singular test (Gauss-Jordan finds
//    no pivot, or |det|^2 < 1e-9, linalg.cpp:23) reports GV_ERR_SINGULAR in
//    info[3] with a zero determinant mantissa, as DetInv sets d = 0; d_Ai
//    then holds whatever the elimination produced and must not be used.
#include <cuda_runtime.h>

#include <mutex>

#include "device.cuh"
#include "kernels.cuh"

namespace gv {
namespace noalloc_detail {

constexpr int kMaxN = GV_NOALLOC_MAX_N;
constexpr int kThreads = 256;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) cx<double> g_noalloc_scratch[kMaxN * kMaxN];

std::mutex g_setup_mutex;
void* g_scratch_address[kMaxDevices] = {};

// The device address of g_noalloc_scratch on the current device (set-up on
// first use per device; host code must not pass the symbol itself).
gv_status scratch_address(cx<double>** out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return GV_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_address[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return GV_ERR_CUDA;
        g_scratch_address[dev] = p;
    }
    *out = static_cast<cx<double>*>(g_scratch_address[dev]);
    return GV_OK;
}

// info[0..3] = det mantissa (re, im), det base-2 exponent, status.
__global__ void __launch_bounds__(kThreads) k_invert_noalloc(const cx<double>* __restrict__ A, cx<double>* Ai, int N,
                                                              cx<double>* M, double* info)
{
    __shared__ __align__(16) char smem[sizeof(cx<double>) * (2 * kMaxN + 2) + sizeof(double) * (kThreads / 32) +
                                       sizeof(int) * (kMaxN + kThreads / 32 + 4) + 64];
    char* p = smem;
    GJSmem S = carve_gj<kThreads>(p, kMaxN);
    for (int idx = threadIdx.x; idx < N * N; idx += kThreads) M[idx] = A[idx];
    __syncthreads();
    cx<double> dm = {0.0, 0.0};
    int de = 0;
    const bool ok = gj_invert<kThreads>(M, N, S, dm, de);
    if (threadIdx.x == 0) { S.detm[0] = dm; S.dete[0] = de; S.flag[0] = ok; }
    __syncthreads();
    dm = S.detm[0];
    de = S.dete[0];
    int status = S.flag[0] ? GV_OK : GV_ERR_SINGULAR;
    if (status == GV_OK) {
        // linalg::DetInv's singular test, |det|^2 < 1e-9 (linalg.cpp:23)
        const double l10 = log10(sqrt(norm2(dm))) + de * 0.30102999566398119521;
        if (2.0 * l10 < -9.0) status = GV_ERR_SINGULAR;
    }
    for (int idx = threadIdx.x; idx < N * N; idx += kThreads) Ai[idx] = M[idx];
    if (threadIdx.x == 0) {
        info[0] = status == GV_OK ? dm.x : 0.0;
        info[1] = status == GV_OK ? dm.y : 0.0;
        info[2] = double(de);
        info[3] = double(status);
    }
}

}  // namespace noalloc_detail
}  // namespace gv

extern "C" gv_status gv_slater_invert_noalloc(const double* d_A, double* d_Ai, int32_t N, double* d_info,
                                              void* stream)
{
    using namespace gv;
    using namespace gv::noalloc_detail;
    if (N < 1 || N > kMaxN) return GV_ERR_TOO_LARGE;
    if (!d_A || !d_Ai || !d_info) return GV_ERR_INVALID;
    if ((reinterpret_cast<uintptr_t>(d_A) | reinterpret_cast<uintptr_t>(d_Ai)) & 15) return GV_ERR_INVALID;
    if (reinterpret_cast<uintptr_t>(d_info) & 7) return GV_ERR_INVALID;   // four doubles written by the kernel
    cx<double>* scratch = nullptr;
    gv_status st = scratch_address(&scratch);
    if (st) return st;
    k_invert_noalloc<<<1, kThreads, 0, static_cast<cudaStream_t>(stream)>>>(
        reinterpret_cast<const cx<double>*>(d_A), reinterpret_cast<cx<double>*>(d_Ai), N, scratch, d_info);
    return cudaGetLastError() == cudaSuccess ? GV_OK : GV_ERR_CUDA;
}
