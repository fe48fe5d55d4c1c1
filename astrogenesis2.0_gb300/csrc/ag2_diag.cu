// ag2_diag.cu -- FP64 diagnostics: direct-summation forces on sampled
// particles (the accuracy oracle of the tree walk), global mass / momentum /
// angular momentum / kinetic energy, and a FP32 FMA throughput probe used as the
// roofline denominator of the walk.
//
// The direct sum uses the reference's softened pair law (Node.cpp:285-305): with
// the integer truncation of abs() the law is G m d / (|d| (|d|^2 + e0^2)) for
// every e0 < 0.66; larger e0 goes through the general law.
#include <vector>

#include "ag2_internal.cuh"

namespace ag2 {

namespace {

constexpr int kDirectBlock = 256;

__device__ double softening_kernel_d(double u)
{
    if (u >= 0 && u < 0.5)
        return (16.0 / 3.0) * (u * u) - (48.0 / 5.0) * pow(u, 4.0) + (32.0 / 5.0) * pow(u, 5.0) - (14.0 / 5.0);
    if (u >= 0.5 && u < 1.0)
        return (1.0 / (15.0 * u)) + (32.0 / 3.0) * (u * u) - 16.0 * pow(u, 3.0) - (48.0 / 5.0) * pow(u, 4.0) -
               (32.0 / 15.0) * pow(u, 5.0) - (16.0 / 5.0);
    if (u >= 1.0) return -1.0 / u;
    return 0.0;
}

// One block per sample: threads stride over all sources, FP64 throughout.
template <bool kGeneral>
__global__ void __launch_bounds__(kDirectBlock) k_direct(const double *__restrict__ px, const double *__restrict__ py,
                                                         const double *__restrict__ pz, const double *__restrict__ m,
                                                         const int32_t *__restrict__ slot, const int32_t *pinst,
                                                         const int64_t *first, double e0, double G,
                                                         double *__restrict__ out)
{
    __shared__ double red[3][kDirectBlock / 32];
    const int s = blockIdx.x;
    const int i = slot[s];
    const int k = pinst[i];
    const int j0 = (int)first[k], n = (int)first[k + 1];  // sources: the sample's own simulation
    const double xi = px[i], yi = py[i], zi = pz[i];
    const double e02 = e0 * e0;
    double ax = 0, ay = 0, az = 0;
    for (int j = j0 + threadIdx.x; j < n; j += blockDim.x) {
        if (j == i) continue;
        double mj = m[j];
        if (mj == 0.0) continue;
        double dx = px[j] - xi, dy = py[j] - yi, dz = pz[j] - zi;
        double r2 = dx * dx + dy * dy + dz * dz;
        if (r2 == 0.0) continue;
        double r = sqrt(r2);
        double eps2 = e02;
        if (kGeneral) {
            double u = r / (2.8 * e0);
            double K = softening_kernel_d(u);
            if ((K - r) == 0) continue;
            double e = -(2.8 * e0) / (K - r);
            if (isnan(e)) continue;
            double ae = (e > -2147483649.0 && e < 2147483648.0) ? fabs(trunc(e)) : -2147483648.0;
            if (ae > e0 * 0.0001 && ae < 1e30) eps2 = e * e;
        }
        double f = G * mj / ((r2 + eps2) * r);
        ax += dx * f;
        ay += dy * f;
        az += dz * f;
    }
    for (int o = 16; o > 0; o >>= 1) {
        ax += __shfl_down_sync(0xffffffffu, ax, o);
        ay += __shfl_down_sync(0xffffffffu, ay, o);
        az += __shfl_down_sync(0xffffffffu, az, o);
    }
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
        red[0][w] = ax;
        red[1][w] = ay;
        red[2][w] = az;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double sx = 0, sy = 0, sz = 0;
        for (int k = 0; k < kDirectBlock / 32; k++) {
            sx += red[0][k];
            sy += red[1][k];
            sz += red[2][k];
        }
        out[3 * s] = sx;
        out[3 * s + 1] = sy;
        out[3 * s + 2] = sz;
    }
}

// slot of each requested caller id
__global__ void k_id_to_slot(int n, const int32_t *id, const int32_t *want, int ns, int32_t *slot)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int o = id[i];
    // want is sorted: binary search
    int lo = 0, hi = ns - 1;
    while (lo <= hi) {
        int mid = (lo + hi) >> 1;
        if (want[mid] == o) {
            slot[mid] = i;
            return;
        }
        if (want[mid] < o)
            lo = mid + 1;
        else
            hi = mid - 1;
    }
}

// per-block partial sums: m, E_kin, p xyz, L xyz
__global__ void k_moments_global(int n, Particles s, double *part)
{
    __shared__ double sh[8][256];
    double v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double m = s.m[i], x = s.px[i], y = s.py[i], z = s.pz[i], vx = s.vx[i], vy = s.vy[i], vz = s.vz[i];
        v[0] += m;
        v[1] += 0.5 * m * (vx * vx + vy * vy + vz * vz);
        v[2] += m * vx;
        v[3] += m * vy;
        v[4] += m * vz;
        v[5] += m * (y * vz - z * vy);
        v[6] += m * (z * vx - x * vz);
        v[7] += m * (x * vy - y * vx);
    }
    for (int k = 0; k < 8; k++) sh[k][threadIdx.x] = v[k];
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w)
            for (int k = 0; k < 8; k++) sh[k][threadIdx.x] += sh[k][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int k = 0; k < 8; k++) part[8 * blockIdx.x + k] = sh[k][0];
}

// FMA throughput probe: 8 independent chains per thread
__global__ void k_fma_probe(float *out, int iters, float a, float b)
{
    float x[8];
    for (int k = 0; k < 8; k++) x[k] = threadIdx.x * 1e-3f + k;
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int k = 0; k < 8; k++) x[k] = fmaf(x[k], a, b);
    }
    float s = 0;
    for (int k = 0; k < 8; k++) s += x[k];
    if (s == 1234.5678f) out[0] = s;  // keeps the chains alive
}

}  // namespace

int run_direct_sum(Ctx *c, size_t ns, const int64_t *ids_host, double *out_host)
{
    const int n = (int)c->n;
    if (ns == 0) return AG2_OK;
    int rc = ensure_instance_tables(c);
    if (rc) return rc;
    if (ns > c->cap) return set_err(c, AG2_E_INVALID, "more samples than particles");
    std::vector<std::pair<int32_t, size_t>> order(ns);
    for (size_t k = 0; k < ns; k++) {
        if (ids_host[k] < 0 || ids_host[k] >= n) return set_err(c, AG2_E_INVALID, "sample id out of range");
        order[k] = {(int32_t)ids_host[k], k};
    }
    std::sort(order.begin(), order.end());
    std::vector<int32_t> want(ns);
    for (size_t k = 0; k < ns; k++) want[k] = order[k].first;
    int32_t *d_want = c->finalnode, *d_slot = c->nodelist;  // scratch (cap entries each)
    double *d_out = c->staging;
    AG2_CUDA(c, cudaMemcpyAsync(d_want, want.data(), ns * 4, cudaMemcpyHostToDevice, c->stream));
    Particles &S = c->S();
    AG2_LAUNCH(c, k_id_to_slot, grid_for(n, 256), 256, 0, n, S.id, d_want, (int)ns, d_slot);
    const bool general = !(c->prm.e0 > 0.0 && c->prm.e0 < 0.6);
    if (general)
        AG2_LAUNCH(c, k_direct<true>, (unsigned)ns, kDirectBlock, 0, S.px, S.py, S.pz, S.m, d_slot, c->pinst,
                   c->inst_first, c->prm.e0, c->prm.G, d_out);
    else
        AG2_LAUNCH(c, k_direct<false>, (unsigned)ns, kDirectBlock, 0, S.px, S.py, S.pz, S.m, d_slot, c->pinst,
                   c->inst_first, c->prm.e0, c->prm.G, d_out);
    std::vector<double> tmp(3 * ns);
    AG2_CUDA(c, cudaMemcpyAsync(tmp.data(), d_out, 3 * ns * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    AG2_CUDA(c, cudaStreamSynchronize(c->stream));
    for (size_t k = 0; k < ns; k++)
        for (int a = 0; a < 3; a++) out_host[3 * order[k].second + a] = tmp[3 * k + a];
    return AG2_OK;
}

int run_diagnostics(Ctx *c, double *out8)
{
    const int n = (int)c->n;
    for (int k = 0; k < 8; k++) out8[k] = 0.0;
    if (n == 0) return AG2_OK;
    const int blocks = 256;
    double *part = c->staging;
    AG2_LAUNCH(c, k_moments_global, blocks, 256, 0, n, c->S(), part);
    std::vector<double> h(8 * blocks);
    AG2_CUDA(c, cudaMemcpyAsync(h.data(), part, h.size() * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    AG2_CUDA(c, cudaStreamSynchronize(c->stream));
    for (int b = 0; b < blocks; b++)
        for (int k = 0; k < 8; k++) out8[k] += h[8 * b + k];
    return AG2_OK;
}

int run_fma_probe(Ctx *c, double *gflops)
{
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
    float *d = reinterpret_cast<float *>(c->staging);
    const int iters = 1 << 16, blocks = sms * 8, threads = 256;
    cudaEvent_t e0, e1;
    AG2_CUDA(c, cudaEventCreate(&e0));
    AG2_CUDA(c, cudaEventCreate(&e1));
    AG2_LAUNCH(c, k_fma_probe, blocks, threads, 0, d, 256, 1.0000001f, 1e-7f);  // warm-up
    AG2_CUDA(c, cudaEventRecord(e0, c->stream));
    AG2_LAUNCH(c, k_fma_probe, blocks, threads, 0, d, iters, 1.0000001f, 1e-7f);
    AG2_CUDA(c, cudaEventRecord(e1, c->stream));
    AG2_CUDA(c, cudaEventSynchronize(e1));
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    double flops = 2.0 * 8.0 * (double)iters * (double)blocks * threads;
    *gflops = flops / (ms * 1e-3) / 1e9;
    return AG2_OK;
}

}  // namespace ag2
