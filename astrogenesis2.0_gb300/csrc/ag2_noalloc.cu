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
// context.  The kernels follow the context path's width rule (sequential sums
// up to 4096 particles, a 64-ary tree of sequential runs above) reading
// xyz-interleaved positions, and give bit-identical results to ag2_build_tree's
// root half-width (ag2_root_radius).  The scratch holds the tree's second level
// (one pair per 4096 particles), which bounds n at AG2_NOALLOC_MAX_PARTICLES.
//
// The scratch array is 32 KiB per device, owned by this library from its first
// use on a device until the process exits.  Every call shares it and leaves
// the previous call's values in it, so calls that overlap on the GPU (on
// different streams, or from different host threads) race; serialise them.
#include <cstdint>
#include <mutex>
#include <tuple>

#include "ag2_internal.cuh"

namespace ag2 {

namespace {

constexpr int kNaBlock = 256;
constexpr int kNaBlocks = 608;        // grid of the max pass
constexpr int kNaSlots = 2040;        // second-level pairs held in the scratch (8,355,840 particles)
constexpr int kNaSeqMax = 4096;       // sequential sums up to this, as the context path
constexpr int kNaMaxDevices = 64;

struct NoAllocScratch {
    double part[2 * kNaSlots];        // second-level sums of |x| and |x|^2 (4096 particles each)
    double sum_d, sum_d2, thr;
    unsigned long long R_bits;        // running max of |x| (bit pattern of a positive double)
};
static_assert(sizeof(NoAllocScratch) <= 32768, "scratch larger than its stated size");

// The scratch itself: a file-scope device array of fixed size.  Host code must
// not pass its name to a kernel (that is a host-side stand-in, not a device
// address); it uses the address obtained with cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[32768];

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

// second level of the 64-ary tree: entry e sums the 64 runs of 64 particles
// starting at particle 4096*e, each run sequentially, the runs in order
__global__ void k_na_level2(const double *pos, int n, int nent, NoAllocScratch *s)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nent) return;
    double a = 0.0, b = 0.0;
    for (int r = 0; r < 64; r++) {
        const int64_t lo = (int64_t)e * 4096 + (int64_t)r * 64;
        if (lo >= n) break;
        const int64_t hi = min(lo + 64, (int64_t)n);
        double ra = 0.0, rb = 0.0;
        for (int64_t q = lo; q < hi; q++) {
            double d = na_dist(pos, (int)q);
            ra = __dadd_rn(ra, d);
            rb = __dadd_rn(rb, __dmul_rn(d, d));
        }
        a = __dadd_rn(a, ra);
        b = __dadd_rn(b, rb);
    }
    s->part[2 * e] = a;
    s->part[2 * e + 1] = b;
}

// remaining levels: runs of 64 pairs, in place, until one pair is left
__global__ void k_na_final(int nent, NoAllocScratch *s)
{
    if (threadIdx.x != 0) return;
    int cnt = nent;
    while (cnt > 1) {
        const int nn = (cnt + 63) / 64;
        for (int j = 0; j < nn; j++) {
            double a = 0.0, b = 0.0;
            for (int q = 64 * j; q < min(64 * j + 64, cnt); q++) {
                a = __dadd_rn(a, s->part[2 * q]);
                b = __dadd_rn(b, s->part[2 * q + 1]);
            }
            s->part[2 * j] = a;
            s->part[2 * j + 1] = b;
        }
        cnt = nn;
    }
    s->sum_d = s->part[0];
    s->sum_d2 = s->part[1];
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

// One launch through cudaLaunchKernel, which returns that launch's status.
// The arguments are converted to the kernel's parameter types first, and the
// launch reads them through pointers before it returns.
template <class... P, class... A>
cudaError_t na_launch(void (*kernel)(P...), int grid, int block, cudaStream_t st, A... args)
{
    std::tuple<P...> t(args...);
    void *pa[sizeof...(P)];
    std::apply([&pa](auto &...x) {
        int i = 0;
        ((pa[i++] = (void *)&x), ...);
    }, t);
    return cudaLaunchKernel((const void *)kernel, dim3(grid), dim3(block), pa, 0, st);
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
    // Each launch's own status comes back from cudaLaunchKernel, so an error
    // that the caller's earlier work left pending is neither consumed nor
    // blamed on this call.  A failed launch of this call stops it, and its
    // error is cleared so that the caller's next cudaGetLastError does not
    // report it a second time.
    auto failed = [](cudaError_t e) {
        if (e == cudaSuccess) return false;
        cudaGetLastError();
        return true;
    };
    if (failed(na_launch(k_na_clear, 1, 32, st, s))) return AG2_E_CUDA;
    if (ni <= kNaSeqMax) {
        if (failed(na_launch(k_na_seq, 1, 1, st, pos, ni, s))) return AG2_E_CUDA;
    } else {
        const int nent = (ni + 4095) / 4096;
        if (failed(na_launch(k_na_level2, (nent + kNaBlock - 1) / kNaBlock, kNaBlock, st, pos, ni, nent, s)))
            return AG2_E_CUDA;
        if (failed(na_launch(k_na_final, 1, 32, st, nent, s))) return AG2_E_CUDA;
    }
    if (failed(na_launch(k_na_thr, 1, 32, st, ni, s))) return AG2_E_CUDA;
    if (failed(na_launch(k_na_max, kNaBlocks, kNaBlock, st, pos, ni, s))) return AG2_E_CUDA;
    if (failed(na_launch(k_na_out, 1, 32, st, (const NoAllocScratch *)s, radius))) return AG2_E_CUDA;
    return AG2_OK;
}
