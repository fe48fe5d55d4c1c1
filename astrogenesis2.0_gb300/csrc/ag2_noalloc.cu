// ag2_noalloc.cu -- root half-width of the octree (Tree::calcTreeWidth,
// simulation/src/Physics/Tree/Tree.cpp:86-117) for callers that cannot allocate
// device memory.
//
// Who needs it: a host integrator that has reserved the GPU's memory for its
// own pools (so that a cudaMalloc here would fail or fragment its budget), and
// code that is in the middle of capturing a CUDA stream, where an allocation
// would break the capture.  Such callers hand in their own device buffers for
// the positions and the result; the per-block partial sums this computation
// needs live in a fixed array in this file instead of in memory allocated by a
// context.  The kernels are copies of the context path's width kernels reading
// xyz-interleaved positions, and give bit-identical results to ag2_build_tree's
// root half-width (ag2_root_radius).
//
// The scratch array is 16 KiB per device, owned by this library from its first
// use on a device until the process exits.  Every call shares it and leaves
// the previous call's values in it, so calls that overlap on the GPU (on
// different streams, or from different host threads) race; serialise them.
#include <mutex>

#include "ag2_internal.cuh"

namespace ag2 {

namespace {

constexpr int kNaBlock = 256;
constexpr int kNaBlocks = 608;        // same fixed grid as the context path
constexpr int kNaSeqMax = 32768;      // sequential sums below this, as the context path
constexpr int kNaMaxDevices = 64;

struct NoAllocScratch {
    double part[2 * kNaBlocks];       // per-block sums of |x| and |x|^2
    double sum_d, sum_d2, thr;
    unsigned long long R_bits;        // running max of |x| (bit pattern of a positive double)
};
static_assert(sizeof(NoAllocScratch) <= 16384, "scratch larger than its stated size");

// The scratch itself: a file-scope device array of fixed size.  Host code must
// not pass its name to a kernel (that is a host-side stand-in, not a device
// address); it uses the address obtained with cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[16384];

std::mutex g_setup_mutex;
void *g_scratch_addr[kNaMaxDevices] = {};

__device__ __forceinline__ double na_dist(const double *pos, int i)
{
    const double x = pos[3 * (size_t)i], y = pos[3 * (size_t)i + 1], z = pos[3 * (size_t)i + 2];
    return sqrt(__dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z)));
}

__global__ void k_na_clear(NoAllocScratch *s)
{
    if (threadIdx.x == 0) {
        s->sum_d = s->sum_d2 = s->thr = 0.0;
        s->R_bits = 0ull;
    }
}

__global__ void k_na_seq(const double *pos, int n, NoAllocScratch *s)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double a = 0.0, b = 0.0;
    for (int i = 0; i < n; i++) {
        double d = na_dist(pos, i);
        a = __dadd_rn(a, d);
        b = __dadd_rn(b, __dmul_rn(d, d));
    }
    s->sum_d = a;
    s->sum_d2 = b;
}

__global__ void k_na_partial(const double *pos, int n, NoAllocScratch *s)
{
    __shared__ double sh[2][kNaBlock];
    double a = 0.0, b = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double d = na_dist(pos, i);
        a += d;
        b += d * d;
    }
    sh[0][threadIdx.x] = a;
    sh[1][threadIdx.x] = b;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            sh[0][threadIdx.x] += sh[0][threadIdx.x + w];
            sh[1][threadIdx.x] += sh[1][threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        s->part[2 * blockIdx.x] = sh[0][0];
        s->part[2 * blockIdx.x + 1] = sh[1][0];
    }
}

__global__ void k_na_final(NoAllocScratch *s)
{
    if (threadIdx.x != 0) return;
    double a = 0.0, b = 0.0;
    for (int k = 0; k < kNaBlocks; k++) {
        a += s->part[2 * k];
        b += s->part[2 * k + 1];
    }
    s->sum_d = a;
    s->sum_d2 = b;
}

__global__ void k_na_thr(int n, NoAllocScratch *s)
{
    if (threadIdx.x != 0) return;
    double mean = s->sum_d / (double)n;
    double sd = sqrt(__dsub_rn(s->sum_d2 / (double)n, __dmul_rn(mean, mean)));
    s->thr = __dadd_rn(mean, __dmul_rn(10.0, sd));
    s->R_bits = 0ull;
}

__global__ void k_na_max(const double *pos, int n, NoAllocScratch *s)
{
    __shared__ unsigned long long sh[kNaBlock];
    const double thr = s->thr;
    unsigned long long best = 0ull;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double d = na_dist(pos, i);
        if (d <= thr && d > 0.0) {
            unsigned long long k = (unsigned long long)__double_as_longlong(d);
            best = k > best ? k : best;
        }
    }
    sh[threadIdx.x] = best;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] = max(sh[threadIdx.x], sh[threadIdx.x + w]);
        __syncthreads();
    }
    if (threadIdx.x == 0 && sh[0] != 0ull) atomicMax(&s->R_bits, sh[0]);
}

__global__ void k_na_out(const NoAllocScratch *s, double *radius)
{
    if (threadIdx.x == 0) radius[0] = __longlong_as_double((long long)s->R_bits);
}

// Device address of the scratch array on the current device, looked up once
// per device.
int scratch_for_current_device(NoAllocScratch **out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNaMaxDevices) return AG2_E_CUDA;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) return AG2_E_CUDA;
        g_scratch_addr[dev] = p;
    }
    *out = reinterpret_cast<NoAllocScratch *>(g_scratch_addr[dev]);
    return AG2_OK;
}

}  // namespace

}  // namespace ag2

extern "C" int ag2_root_radius_noalloc(const double *pos, int64_t n, double *radius, void *stream)
{
    using namespace ag2;
    if (!pos || !radius || n < 1) return AG2_E_INVALID;
    if (n > (int64_t)AG2_NOALLOC_MAX_PARTICLES) return AG2_E_CAPACITY;
    NoAllocScratch *s = nullptr;
    int rc = scratch_for_current_device(&s);
    if (rc != AG2_OK) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const int ni = (int)n;
    k_na_clear<<<1, 32, 0, st>>>(s);
    if (ni <= kNaSeqMax) {
        k_na_seq<<<1, 1, 0, st>>>(pos, ni, s);
    } else {
        k_na_partial<<<kNaBlocks, kNaBlock, 0, st>>>(pos, ni, s);
        k_na_final<<<1, 32, 0, st>>>(s);
    }
    k_na_thr<<<1, 32, 0, st>>>(ni, s);
    k_na_max<<<kNaBlocks, kNaBlock, 0, st>>>(pos, ni, s);
    k_na_out<<<1, 32, 0, st>>>(s, radius);
    return cudaGetLastError() == cudaSuccess ? AG2_OK : AG2_E_CUDA;
}
