// ag2_io.cu -- snapshot files and initial conditions, encoded and decoded on
// the device.
//
// The reference's DataManager packs Particle objects into byte records one
// memcpy at a time (saveData, File/DataManager.cpp:86-424) and unpacks them the
// same way (loadICs, :434-1332).  Here the file image lives in HBM:
//   * ag / agc / age records: a warp assembles 32 consecutive records in shared
//     memory and moves the chunk with 8-byte coalesced stores or loads.  Every
//     chunk starts 8-byte aligned (the 40-byte header plus 32 records of 62, 26
//     or 94 bytes), and every record length is even, so records are packed in
//     16-bit pieces.
//   * gadget: the writer's particle lists are a stable three-way partition
//     (per-block counts, one scan block, ranks from warp ballots), each
//     particle writes its floats at its list position.
//   * one copy moves the image between HBM and pinned host memory; a snapshot
//     file is written by a background thread while the device moves on.
// The state arrays are in tree order; files are in upload order, through the
// inverse of Particles::id.
#include <cstdio>
#include <cstring>

#include "ag2_internal.cuh"

namespace ag2 {

int upload_common(Ctx *c, size_t n, const double *pos, const double *vel, const double *mass, const double *U,
                  const uint8_t *type);

namespace {

constexpr int kIoBlock = 256;
constexpr int kGadBlock = 1024;
constexpr int kHdr = 40;        // AGFHeader: int numParticles[3], 4 padding bytes, 3 doubles (DataManager.h:44-50)
constexpr size_t kSlack = 64;   // device image slack: the last chunk's word tail may run past the end
// Units.h:6-20
constexpr double kKpc = 3.08567758149137e19;
constexpr double kKms = 1.0e3;
constexpr double kMsun = 1.98847e30;
constexpr double kMassUnit = kMsun * 1e10;  // Units::MSUN * 1e10 (DataManager.cpp:398)
// the gadget writer's prepareData takes its unit as a float (DataManager.cpp:322)
constexpr double kKpcF = (double)(float)kKpc;
constexpr double kKmsF = (double)(float)kKms;

__host__ __device__ constexpr int rec_bytes(int fmt)
{
    return fmt == AG2_FMT_AG ? 62 : fmt == AG2_FMT_AGC ? 26 : 94;
}

// ---- 16-bit packing of a record in shared memory (little endian) ----------
__device__ inline void put32(uint16_t *r, int off, uint32_t b)
{
    r[off / 2] = (uint16_t)b;
    r[off / 2 + 1] = (uint16_t)(b >> 16);
}
__device__ inline void put64(uint16_t *r, int off, double v)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    put32(r, off, (uint32_t)b);
    put32(r, off + 4, (uint32_t)(b >> 32));
}
__device__ inline void putf(uint16_t *r, int off, double v) { put32(r, off, __float_as_uint(__double2float_rn(v))); }
__device__ inline uint32_t get32(const uint16_t *r, int off) { return r[off / 2] | ((uint32_t)r[off / 2 + 1] << 16); }
__device__ inline double get64(const uint16_t *r, int off)
{
    return __longlong_as_double((long long)(get32(r, off) | ((unsigned long long)get32(r, off + 4) << 32)));
}
__device__ inline double getf(const uint16_t *r, int off) { return (double)__uint_as_float(get32(r, off)); }

__global__ void k_inverse(int n, const int32_t *__restrict__ id, int32_t *__restrict__ inv)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) inv[id[i]] = i;
}

// saveData's ag / agc / age records (DataManager.cpp:120-258) of upload
// indices [0, count); tcount[0..2] += particles of type 1, 2, 3.
template <int kFmt>
__global__ void __launch_bounds__(kIoBlock) k_snap_records(int64_t count, Particles s, const int32_t *__restrict__ inv,
                                                           const uint32_t *__restrict__ tid,
                                                           const uint8_t *__restrict__ tgp,
                                                           const double *__restrict__ tsfr, uint8_t *img,
                                                           int32_t *tcount)
{
    constexpr int R = rec_bytes(kFmt);
    __shared__ __align__(8) uint16_t sm[kIoBlock / 32][32 * R / 2];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t base = (int64_t)blockIdx.x * kIoBlock + w * 32;
    if (base >= count) return;  // whole warps only
    const int64_t o = base + lane;
    const bool valid = o < count;
    uint16_t *r = sm[w] + lane * (R / 2);
    int ty = 0;
    if (valid) {
        const int i = inv[o];
        ty = s.type[i];
        const uint16_t tg = (uint16_t)(ty | (tgp[o] << 8));
        if (kFmt == AG2_FMT_AGC) {
            putf(r, 0, s.px[i]);
            putf(r, 4, s.py[i]);
            putf(r, 8, s.pz[i]);
            putf(r, 12, s.vdens[i]);
            putf(r, 16, tsfr[o]);
            putf(r, 20, s.T[i]);
            r[12] = tg;
        } else if (kFmt == AG2_FMT_AG) {
            put64(r, 0, s.px[i]);
            put64(r, 8, s.py[i]);
            put64(r, 16, s.pz[i]);
            put64(r, 24, s.m[i]);
            put64(r, 32, s.T[i]);
            put64(r, 40, s.vdens[i]);
            put64(r, 48, tsfr[o]);
            r[28] = tg;
            put32(r, 58, tid[o]);
        } else {
            put64(r, 0, s.px[i]);
            put64(r, 8, s.py[i]);
            put64(r, 16, s.pz[i]);
            put64(r, 24, s.vx[i]);
            put64(r, 32, s.vy[i]);
            put64(r, 40, s.vz[i]);
            put64(r, 48, s.m[i]);
            put64(r, 56, s.T[i]);
            put64(r, 64, s.P[i]);
            put64(r, 72, s.vdens[i]);
            put64(r, 80, s.U[i]);
            r[44] = tg;
            put32(r, 90, tid[o]);
        }
    }
    const unsigned b1 = __ballot_sync(~0u, ty == 1), b2 = __ballot_sync(~0u, ty == 2), b3 = __ballot_sync(~0u, ty == 3);
    if (lane == 0) {
        if (b1) atomicAdd(&tcount[0], __popc(b1));
        if (b2) atomicAdd(&tcount[1], __popc(b2));
        if (b3) atomicAdd(&tcount[2], __popc(b3));
    }
    __syncwarp();
    const int64_t nrec = count - base < 32 ? count - base : 32;
    const int nwords = (int)((nrec * R + 7) / 8);
    unsigned long long *dst = reinterpret_cast<unsigned long long *>(img + kHdr + base * R);
    const unsigned long long *src = reinterpret_cast<const unsigned long long *>(sm[w]);
    for (int k = lane; k < nwords; k += 32) dst[k] = src[k];
}

// AGFHeader (DataManager.cpp:122-140): numParticles of types 1, 2, 3, then
// deltaTime, endTime, currentTime.  The padding after the counts is zero.
__global__ void k_snap_header(const int32_t *tcount, double dt, double end_time, double t, uint8_t *img)
{
    int32_t *h = reinterpret_cast<int32_t *>(img);
    h[0] = tcount[0];
    h[1] = tcount[1];
    h[2] = tcount[2];
    h[3] = 0;
    double *d = reinterpret_cast<double *>(img + 16);
    d[0] = dt;
    d[1] = end_time;
    d[2] = t;
}

// ---- gadget writer (DataManager.cpp:263-416) --------------------------------
// Classes of a particle by (type, galaxyPart): A disk star (1, 1), B halo dark
// matter (3, 3), C bulge star (1, 2), D gas (2, any), E anything else.  The
// reference collects A and D in "gas_particles", C in "halo_particles" and B in
// "disk_particles" and writes them in that order, so the lists are L0 = A+D,
// L1 = C, L2 = B; E is counted in the header (npart[0]) but written nowhere.
__device__ inline int gad_class(int ty, int gp)
{
    if (ty == 2) return 3;
    if (ty == 1 && gp == 1) return 0;
    if (ty == 3 && gp == 3) return 1;
    if (ty == 1 && gp == 2) return 2;
    return 4;
}
__device__ inline int class_list(int k) { return k == 0 || k == 3 ? 0 : k == 2 ? 1 : k == 1 ? 2 : -1; }

__global__ void __launch_bounds__(kGadBlock) k_gad_count(int64_t count, const uint8_t *__restrict__ type,
                                                         const int32_t *__restrict__ inv,
                                                         const uint8_t *__restrict__ tgp, int32_t *bc)
{
    __shared__ int32_t cnt[5];
    if (threadIdx.x < 5) cnt[threadIdx.x] = 0;
    __syncthreads();
    const int64_t o = (int64_t)blockIdx.x * kGadBlock + threadIdx.x;
    const int k = o < count ? gad_class(type[inv[o]], tgp[o]) : -1;
    for (int q = 0; q < 5; q++) {
        const unsigned b = __ballot_sync(~0u, k == q);
        if ((threadIdx.x & 31) == 0 && b) atomicAdd(&cnt[q], __popc(b));
    }
    __syncthreads();
    if (threadIdx.x < 5) bc[blockIdx.x * 5 + threadIdx.x] = cnt[threadIdx.x];
}

__device__ inline void st32(uint8_t *img, int64_t off, uint32_t v) { *reinterpret_cast<uint32_t *>(img + off) = v; }

// Exclusive scan of the three list counts over the blocks (boff[3b + L]),
// list totals (tot[0..2]), then the header, block markers and image length.
__global__ void __launch_bounds__(kGadBlock) k_gad_scan(int nb, const int32_t *__restrict__ bc, int32_t *boff,
                                                        int32_t *tot, double t, uint8_t *img, int64_t *len)
{
    __shared__ int32_t wsum[32][3];
    __shared__ int64_t carry[3], cls[5];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (threadIdx.x < 3) carry[threadIdx.x] = 0;
    if (threadIdx.x < 5) cls[threadIdx.x] = 0;
    __syncthreads();
    for (int b0 = 0; b0 < nb; b0 += kGadBlock) {
        const int b = b0 + threadIdx.x;
        int v[3] = {0, 0, 0}, x[3];
        if (b < nb) {
            const int32_t *q = bc + 5 * b;
            v[0] = q[0] + q[3];
            v[1] = q[2];
            v[2] = q[1];
            for (int k = 0; k < 5; k++)
                if (q[k]) atomicAdd(reinterpret_cast<unsigned long long *>(&cls[k]), (unsigned long long)q[k]);
        }
        for (int L = 0; L < 3; L++) {
            int s = v[L];
            for (int d = 1; d < 32; d <<= 1) {
                const int y = __shfl_up_sync(~0u, s, d);
                if (lane >= d) s += y;
            }
            x[L] = s - v[L];
            if (lane == 31) wsum[w][L] = s;
        }
        __syncthreads();
        for (int L = 0; L < 3; L++) {
            int pre = 0;
            for (int k = 0; k < w; k++) pre += wsum[k][L];
            if (b < nb) boff[3 * b + L] = (int32_t)(carry[L] + pre + x[L]);
        }
        __syncthreads();
        if (threadIdx.x < 3) {
            int64_t s = 0;
            for (int k = 0; k < 32; k++) s += wsum[k][threadIdx.x];
            carry[threadIdx.x] += s;
        }
        __syncthreads();
    }
    if (threadIdx.x != 0) return;
    for (int L = 0; L < 3; L++) tot[L] = (int32_t)carry[L];
    const int64_t M = carry[0] + carry[1] + carry[2], G = carry[0];
    // gadget2Header (DataManager.h:53-74), zero but for the fields saveData sets
    for (int k = 0; k < 264; k += 4) st32(img, k, 0u);
    st32(img, 0, 256u);
    st32(img, 260, 256u);
    const uint32_t npart[6] = {(uint32_t)(cls[3] + cls[4]), (uint32_t)cls[1], (uint32_t)cls[0], (uint32_t)cls[2], 0u, 0u};
    for (int k = 0; k < 6; k++) {
        st32(img, 4 + 4 * k, npart[k]);   // npart
        st32(img, 100 + 4 * k, npart[k]); // npartTotal
    }
    const unsigned long long tb = (unsigned long long)__double_as_longlong(t);
    st32(img, 4 + 72, (uint32_t)tb);  // time
    st32(img, 4 + 76, (uint32_t)(tb >> 32));
    st32(img, 4 + 124, 1u);  // num_files
    const unsigned long long hb = (unsigned long long)__double_as_longlong(1.0);
    st32(img, 4 + 152, (uint32_t)hb);  // HubbleParam
    st32(img, 4 + 156, (uint32_t)(hb >> 32));
    int64_t p = 264;
    const int64_t bytes[5] = {12 * M, 12 * M, 4 * M, 4 * M, 4 * G};
    for (int k = 0; k < 5; k++) {
        if (k == 4 && G == 0) break;
        st32(img, p, (uint32_t)bytes[k]);
        st32(img, p + 4 + bytes[k], (uint32_t)bytes[k]);
        p += 8 + bytes[k];
    }
    *len = p;
}

__global__ void __launch_bounds__(kGadBlock) k_gad_write(int64_t count, Particles s, const int32_t *__restrict__ inv,
                                                         const uint32_t *__restrict__ tid,
                                                         const uint8_t *__restrict__ tgp,
                                                         const int32_t *__restrict__ boff,
                                                         const int32_t *__restrict__ tot, uint8_t *img)
{
    __shared__ int32_t wcnt[32][3];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t o = (int64_t)blockIdx.x * kGadBlock + threadIdx.x;
    const int i = o < count ? inv[o] : 0;
    const int L = o < count ? class_list(gad_class(s.type[i], tgp[o])) : -1;
    int rank = 0;
    for (int q = 0; q < 3; q++) {
        const unsigned b = __ballot_sync(~0u, L == q);
        if (L == q) rank = __popc(b & ((1u << lane) - 1u));
        if (lane == 0) wcnt[w][q] = __popc(b);
    }
    __syncthreads();
    if (L < 0) return;
    for (int k = 0; k < w; k++) rank += wcnt[k][L];
    const int64_t T0 = tot[0], T1 = tot[1], M = T0 + T1 + tot[2];
    const int64_t start = L == 0 ? 0 : L == 1 ? T0 : T0 + T1;
    const int64_t q = start + boff[3 * blockIdx.x + L] + rank;
    const int64_t pos_d = 268, vel_d = pos_d + 12 * M + 8, id_d = vel_d + 12 * M + 8, mass_d = id_d + 4 * M + 8,
                  u_d = mass_d + 4 * M + 8;
    float *pf = reinterpret_cast<float *>(img + pos_d) + 3 * q;
    float *vf = reinterpret_cast<float *>(img + vel_d) + 3 * q;
    const double x = s.px[i], y = s.py[i], z = s.pz[i];
    pf[0] = __double2float_rn(x / kKpcF);
    pf[1] = __double2float_rn(y / kKpcF);
    pf[2] = __double2float_rn(z / kKpcF);
    // the reference's velocity block holds position / Units::KMS
    // (prepareData reads position, DataManager.cpp:322-329 with :349-356)
    vf[0] = __double2float_rn(x / kKmsF);
    vf[1] = __double2float_rn(y / kKmsF);
    vf[2] = __double2float_rn(z / kKmsF);
    reinterpret_cast<uint32_t *>(img + id_d)[q] = tid[o];
    reinterpret_cast<float *>(img + mass_d)[q] = __double2float_rn(s.m[i] / kMassUnit);
    if (L == 0) reinterpret_cast<float *>(img + u_d)[q] = __double2float_rn(s.U[i] / 1e6);
}

// ---- loaders ----------------------------------------------------------------
struct IcOut {
    double *pos, *vel, *m, *U, *T, *P, *vd;
    uint8_t *type;
    uint32_t *tid;
    uint8_t *tgp;
    double *tsfr;
};

// loadICs ag / agc / age (DataManager.cpp:446-573): records in file order
template <int kFmt>
__global__ void __launch_bounds__(kIoBlock) k_ic_records(int64_t n, const uint8_t *__restrict__ img, IcOut out)
{
    constexpr int R = rec_bytes(kFmt);
    __shared__ __align__(8) uint16_t sm[kIoBlock / 32][32 * R / 2];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t base = (int64_t)blockIdx.x * kIoBlock + w * 32;
    if (base >= n) return;
    const int64_t nrec = n - base < 32 ? n - base : 32;
    const int nwords = (int)((nrec * R + 7) / 8);
    const unsigned long long *src = reinterpret_cast<const unsigned long long *>(img + kHdr + base * R);
    unsigned long long *dst = reinterpret_cast<unsigned long long *>(sm[w]);
    for (int k = lane; k < nwords; k += 32) dst[k] = src[k];
    __syncwarp();
    const int64_t o = base + lane;
    if (o >= n) return;
    const uint16_t *r = sm[w] + lane * (R / 2);
    if (kFmt == AG2_FMT_AGC) {
        out.pos[3 * o] = getf(r, 0);
        out.pos[3 * o + 1] = getf(r, 4);
        out.pos[3 * o + 2] = getf(r, 8);
        out.vd[o] = getf(r, 12);
        out.tsfr[o] = getf(r, 16);
        out.T[o] = getf(r, 20);
        out.type[o] = (uint8_t)r[12];
        out.tgp[o] = (uint8_t)(r[12] >> 8);
        out.tid[o] = (uint32_t)o;  // agc holds no id (the reference leaves Particle::id unset)
        out.m[o] = 0.0;
    } else if (kFmt == AG2_FMT_AG) {
        out.pos[3 * o] = get64(r, 0);
        out.pos[3 * o + 1] = get64(r, 8);
        out.pos[3 * o + 2] = get64(r, 16);
        out.m[o] = get64(r, 24);
        out.T[o] = get64(r, 32);
        out.vd[o] = get64(r, 40);
        out.tsfr[o] = get64(r, 48);
        out.type[o] = (uint8_t)r[28];
        out.tgp[o] = (uint8_t)(r[28] >> 8);
        out.tid[o] = get32(r, 58);
    } else {
        out.pos[3 * o] = get64(r, 0);
        out.pos[3 * o + 1] = get64(r, 8);
        out.pos[3 * o + 2] = get64(r, 16);
        out.vel[3 * o] = get64(r, 24);
        out.vel[3 * o + 1] = get64(r, 32);
        out.vel[3 * o + 2] = get64(r, 40);
        out.m[o] = get64(r, 48);
        out.T[o] = get64(r, 56);
        out.P[o] = get64(r, 64);
        out.vd[o] = get64(r, 72);
        out.U[o] = get64(r, 80);
        out.type[o] = (uint8_t)r[44];
        out.tgp[o] = (uint8_t)(r[44] >> 8);
        out.tid[o] = get32(r, 90);
        out.tsfr[o] = 0.0;
    }
}

// Byte regions of a gadget / makeGal file that the reference reads into its
// arrays.  A region's bytes past `len` read as zero (the reference's arrays
// are zero-initialised and a short block leaves their tails alone).
struct Region {
    int64_t off, len;
};
struct GadLayout {
    int64_t n;
    int64_t type_end[6];   // cumulative particle counts per Gadget type
    Region pos, vel, id, mass, u;
    double hmass[6];       // mass of a type without individual masses, in kg
    int64_t mass_base[6];  // makeGal: index of the type's first value in the mass stream (-1: header mass)
    int mass_mode;         // 0 header masses, 1 gadget mass block (index = particle), 2 makeGal typelist
    int has_u;
    int makegal;
};

__device__ inline uint32_t ld32(const uint8_t *img, const Region &g, int64_t rel)
{
    const int64_t a = g.off + rel;
    if (rel + 4 <= g.len && (a & 3) == 0) return *reinterpret_cast<const uint32_t *>(img + a);
    uint32_t v = 0;
    for (int k = 0; k < 4; k++)
        if (rel + k < g.len) v |= (uint32_t)img[a + k] << (8 * k);
    return v;
}
__device__ inline double ldf(const uint8_t *img, const Region &g, int64_t rel)
{
    return (double)__uint_as_float(ld32(img, g, rel));
}

// loadICs gadget (DataManager.cpp:811-1322) and makeGal (:580-809)
__global__ void k_ic_gadget(GadLayout L, const uint8_t *__restrict__ img, IcOut out)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= L.n) return;
    int t = 0;
    while (t < 5 && i >= L.type_end[t]) t++;
    const int64_t t0 = t ? L.type_end[t - 1] : 0;
    for (int c = 0; c < 3; c++) {
        out.pos[3 * i + c] = ldf(img, L.pos, 12 * i + 4 * c) * kKpc;
        out.vel[3 * i + c] = ldf(img, L.vel, 12 * i + 4 * c) * kKms;
    }
    out.tid[i] = ld32(img, L.id, 4 * i);
    double m;
    if (L.mass_mode == 1) m = ldf(img, L.mass, 4 * i) * kMsun * 1e10;
    else if (L.mass_mode == 2 && L.mass_base[t] >= 0) m = ldf(img, L.mass, 4 * (L.mass_base[t] + i - t0)) * kMsun * 1e10;
    else m = L.hmass[t];
    out.m[i] = m;
    out.U[i] = (L.has_u && t == 0) ? ldf(img, L.u, 4 * i) * 1e6 : 0.0;
    // Gadget type -> (type, galaxyPart): gas, halo, disk, bulge, stars, black
    // holes.  The gadget reader leaves galaxyPart at its default 1 for types
    // 2, 4, 5; makeGal puts type 5 into the bulge.
    const uint8_t ty[6] = {2, 3, 1, 1, 1, 1};
    const uint8_t gp[6] = {1, 3, 1, 2, 1, (uint8_t)(L.makegal ? 2 : 1)};
    out.type[i] = ty[t];
    out.tgp[i] = gp[t];
    out.tsfr[i] = 0.0;
}

// T, P and visualDensity from the loader's scratch (upload order) into the
// freshly uploaded state (slot i holds upload index s.id[i])
__global__ void k_ic_fields(int64_t n, const double *T, const double *P, const double *vd, Particles s)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int u = s.id[i];
    s.T[i] = T[u];
    if (P) s.P[i] = P[u];
    s.vdens[i] = vd[u];
}

__global__ void k_tags_reset(int64_t n, uint32_t *tid, uint8_t *tgp, double *tsfr)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    tid[i] = (uint32_t)i;
    tgp[i] = 1;
    tsfr[i] = 0.0;
}

// ---- host helpers -------------------------------------------------------------
void io_join(Ctx *c)
{
    if (c->io_thread.joinable()) c->io_thread.join();
}

int ensure_io(Ctx *c, size_t dev_bytes, size_t host_bytes, size_t scratch_ints)
{
    if (dev_bytes + kSlack > c->io_dev_cap) {
        if (c->io_dev) cudaFree(c->io_dev);
        c->io_dev = nullptr;
        c->io_dev_cap = 0;
        const size_t cap = dev_bytes + dev_bytes / 8 + kSlack;
        if (cudaMalloc(&c->io_dev, cap) != cudaSuccess) return set_err(c, AG2_E_NOMEM, "file image allocation failed");
        c->io_dev_cap = cap;
    }
    if (host_bytes > c->io_host_cap) {
        if (c->io_host) cudaFreeHost(c->io_host);
        c->io_host = nullptr;
        c->io_host_cap = 0;
        const size_t cap = host_bytes + host_bytes / 8 + 64;
        if (cudaMallocHost(&c->io_host, cap) != cudaSuccess) return set_err(c, AG2_E_NOMEM, "pinned file buffer allocation failed");
        c->io_host_cap = cap;
    }
    if (scratch_ints > c->io_scratch_cap) {
        if (c->io_scratch) cudaFree(c->io_scratch);
        c->io_scratch = nullptr;
        c->io_scratch_cap = 0;
        if (cudaMalloc(&c->io_scratch, scratch_ints * sizeof(int32_t)) != cudaSuccess)
            return set_err(c, AG2_E_NOMEM, "file scratch allocation failed");
        c->io_scratch_cap = scratch_ints;
    }
    if (!c->io_len_dev) {
        if (cudaMalloc(&c->io_len_dev, sizeof(int64_t)) != cudaSuccess ||
            cudaMallocHost(&c->io_len_host, sizeof(int64_t)) != cudaSuccess)
            return set_err(c, AG2_E_NOMEM, "file length allocation failed");
    }
    if (!c->io_stream) {
        AG2_CUDA(c, cudaStreamCreateWithFlags(&c->io_stream, cudaStreamNonBlocking));
        AG2_CUDA(c, cudaEventCreateWithFlags(&c->io_event, cudaEventDisableTiming));
    }
    return AG2_OK;
}

size_t snapshot_bound(int fmt, int64_t count)
{
    if (fmt == AG2_FMT_GADGET) return 304 + 36 * (size_t)count;
    return kHdr + (size_t)count * rec_bytes(fmt);
}

bool writable_format(int fmt) { return fmt >= AG2_FMT_AG && fmt <= AG2_FMT_GADGET; }

// Encode the image of the first `count` particles into c->io_dev (and the
// gadget length into c->io_len_dev).
int encode_snapshot(Ctx *c, int fmt, int64_t count, double dt, double end_time, double t)
{
    const int64_t nb = (count + kGadBlock - 1) / kGadBlock;
    const size_t bound = snapshot_bound(fmt, count);
    int rc = ensure_io(c, bound, 0, c->n + 8 * (size_t)nb + 64);
    if (rc) return rc;
    Particles s = c->S();
    int32_t *inv = c->io_scratch, *small = c->io_scratch + c->n;  // small: 3 type counts / 3 list totals
    int32_t *bc = small + 8, *boff = bc + 5 * nb;
    AG2_LAUNCH(c, k_inverse, grid_for(c->n, kIoBlock), kIoBlock, 0, (int)c->n, s.id, inv);
    if (fmt == AG2_FMT_GADGET) {
        AG2_LAUNCH(c, k_gad_count, (unsigned)nb, kGadBlock, 0, count, s.type, inv, c->tag_gp, bc);
        AG2_LAUNCH(c, k_gad_scan, 1, kGadBlock, 0, (int)nb, bc, boff, small, t, c->io_dev, c->io_len_dev);
        AG2_LAUNCH(c, k_gad_write, (unsigned)nb, kGadBlock, 0, count, s, inv, c->tag_id, c->tag_gp, boff, small,
                   c->io_dev);
        return AG2_OK;
    }
    AG2_CUDA(c, cudaMemsetAsync(small, 0, 3 * sizeof(int32_t), c->stream));
    const unsigned g = grid_for(count, kIoBlock);
    if (fmt == AG2_FMT_AG)
        AG2_LAUNCH(c, k_snap_records<AG2_FMT_AG>, g, kIoBlock, 0, count, s, inv, c->tag_id, c->tag_gp, c->tag_sfr,
                   c->io_dev, small);
    else if (fmt == AG2_FMT_AGC)
        AG2_LAUNCH(c, k_snap_records<AG2_FMT_AGC>, g, kIoBlock, 0, count, s, inv, c->tag_id, c->tag_gp, c->tag_sfr,
                   c->io_dev, small);
    else
        AG2_LAUNCH(c, k_snap_records<AG2_FMT_AGE>, g, kIoBlock, 0, count, s, inv, c->tag_id, c->tag_gp, c->tag_sfr,
                   c->io_dev, small);
    AG2_LAUNCH(c, k_snap_header, 1, 1, 0, small, dt, end_time, t, c->io_dev);
    return AG2_OK;
}

int check_snapshot_args(Ctx *c, int fmt, int64_t count)
{
    if (!writable_format(fmt)) return set_err(c, AG2_E_FORMAT, "unknown snapshot format");
    if (count < 0 || (size_t)count > c->n) return set_err(c, AG2_E_INVALID, "count outside 0..particles");
    if (c->capturing) return set_err(c, AG2_E_INVALID, "snapshot during a stream capture");
    return AG2_OK;
}

// ---- file parsing (host) --------------------------------------------------------
struct IcFile {
    std::vector<uint8_t> small;  // header bytes for ag2_ic_count
    size_t size = 0;
};

uint32_t rd_u32(const uint8_t *b, size_t off)
{
    uint32_t v;
    std::memcpy(&v, b + off, 4);
    return v;
}
int32_t rd_i32(const uint8_t *b, size_t off)
{
    int32_t v;
    std::memcpy(&v, b + off, 4);
    return v;
}
double rd_f64(const uint8_t *b, size_t off)
{
    double v;
    std::memcpy(&v, b + off, 8);
    return v;
}

struct Parsed {
    int fmt = 0;
    int64_t n = 0;
    double times[3] = {0, 0, 0};
    GadLayout g = {};
};

// Parse the structure of a file image b[0, size) the way the reference's
// reader walks it.  Returns AG2_OK, or AG2_E_FORMAT with a message where the
// reference returns false, would overflow an array or reads particle data
// past the end of the file.
int parse_ics(const uint8_t *b, size_t size, int fmt, Parsed &P, std::string &why)
{
    P.fmt = fmt;
    if (fmt == AG2_FMT_AG || fmt == AG2_FMT_AGC || fmt == AG2_FMT_AGE) {
        if (size < (size_t)kHdr) return why = "file shorter than the 40-byte header", AG2_E_FORMAT;
        const int32_t a = rd_i32(b, 0), b1 = rd_i32(b, 4), c = rd_i32(b, 8);
        if (a < 0 || b1 < 0 || c < 0) return why = "negative particle count in the header", AG2_E_FORMAT;
        P.n = (int64_t)a + b1 + c;
        for (int k = 0; k < 3; k++) P.times[k] = rd_f64(b, 16 + 8 * k);
        if ((size_t)kHdr + (size_t)P.n * rec_bytes(fmt) > size)
            return why = "file ends inside the particle records", AG2_E_FORMAT;
        return AG2_OK;
    }
    GadLayout &g = P.g;
    g = GadLayout{};
    if (fmt == AG2_FMT_GADGET) {
        // gadget2Header between two 4-byte block markers (DataManager.cpp:817-843)
        if (size < 264) return why = "file shorter than the gadget header", AG2_E_FORMAT;
        if (rd_u32(b, 0) != 256) return why = "gadget header block size is not 256", AG2_E_FORMAT;
        const uint8_t *h = b + 4;
        uint64_t n = 0;
        uint32_t np[6];
        double massarr[6];
        for (int k = 0; k < 6; k++) {
            np[k] = rd_u32(h, 4 * k);
            massarr[k] = rd_f64(h, 24 + 8 * k);
            n += np[k];
        }
        P.times[2] = rd_f64(h, 72);
        if (n > 0xFFFFFFFFull) return why = "particle count overflows 32 bits", AG2_E_FORMAT;
        P.n = (int64_t)n;
        int64_t acc = 0;
        for (int k = 0; k < 6; k++) g.type_end[k] = acc += np[k];
        // has_individual_mass (DataManager.cpp:975-993): a type with particles
        // and massarr below 1e-10f
        const double eps = (double)1e-10f;
        bool ind = false;
        for (int k = 0; k < 6; k++)
            if (massarr[k] < eps && np[k] != 0) {
                ind = true;
                break;
            }
        size_t p = 264;
        auto block = [&](Region &r, uint64_t expected, const char *name) -> int {
            if (p + 4 > size) return why = std::string("file ends before the ") + name + " block", AG2_E_FORMAT;
            const uint32_t bs = rd_u32(b, p);
            if (bs > expected) return why = std::string(name) + " block larger than its particles", AG2_E_FORMAT;
            if (p + 8 + (size_t)bs > size) return why = std::string("file ends inside the ") + name + " block", AG2_E_FORMAT;
            if (rd_u32(b, p + 4 + bs) != bs) return why = std::string(name) + " block markers differ", AG2_E_FORMAT;
            r = Region{(int64_t)p + 4, (int64_t)bs};
            p += 8 + bs;
            return AG2_OK;
        };
        int rc;
        if ((rc = block(g.pos, 12 * n, "POS")) || (rc = block(g.vel, 12 * n, "VEL")) || (rc = block(g.id, 4 * n, "ID")))
            return rc;
        if (ind) {
            if ((rc = block(g.mass, 4 * n, "MASS"))) return rc;
            g.mass_mode = 1;
        }
        if (np[0] > 0) {
            if ((rc = block(g.u, 4ull * np[0], "U"))) return rc;
            g.has_u = 1;
        }
        for (int k = 0; k < 6; k++) g.hmass[k] = massarr[k] * kMsun * 1e10;
        g.n = P.n;
        return AG2_OK;
    }
    if (fmt != AG2_FMT_MAKEGAL) return why = "unknown initial-condition format", AG2_E_FORMAT;
    // makeGal (DataManager.cpp:580-650): a 16-byte label record, the header
    // record, then for POS, VEL, ID, MASS, U each a label record, a 4-byte
    // size, the values the reader consumes and a 4-byte trailer.  The reader
    // consumes a fixed number of bytes per block whatever the file's sizes say.
    if (size < 280) return why = "file shorter than the makeGal header", AG2_E_FORMAT;
    const uint8_t *h = b + 20;
    int64_t n = 0;
    int32_t np[6];
    double mass[6];
    for (int k = 0; k < 6; k++) {
        np[k] = rd_i32(h, 4 * k);
        mass[k] = rd_f64(h, 24 + 8 * k);
        if (np[k] < 0) return why = "negative particle count in the header", AG2_E_FORMAT;
        n += np[k];
    }
    P.times[2] = rd_f64(h, 72);
    P.n = n;
    int64_t acc = 0, K = 0;
    for (int k = 0; k < 6; k++) {
        g.type_end[k] = acc += np[k];
        const bool individual = mass[k] == 0 && np[k] > 0;  // typelist (DataManager.cpp:678-683)
        g.mass_base[k] = individual ? K : -1;
        if (individual) K += np[k];
        g.hmass[k] = (double)(float)mass[k] * kMsun * 1e10;
    }
    size_t p = 280;
    Region *regs[5] = {&g.pos, &g.vel, &g.id, &g.mass, &g.u};
    const int64_t bytes[5] = {12 * n, 12 * n, 4 * n, 4 * K, 4 * (int64_t)np[0]};
    for (int k = 0; k < 5; k++) {
        p += 16 + 4;
        *regs[k] = Region{(int64_t)p, bytes[k]};
        p += bytes[k] + 4;
    }
    if ((size_t)(g.u.off + g.u.len) > size) return why = "file ends inside the particle data", AG2_E_FORMAT;
    g.mass_mode = 2;
    g.has_u = 1;
    g.makegal = 1;
    g.n = n;
    return AG2_OK;
}

int read_file(const char *path, std::vector<uint8_t> *small, uint8_t **pinned, size_t *size, Ctx *c)
{
    FILE *f = std::fopen(path, "rb");
    if (!f) return AG2_E_IO;
    std::fseek(f, 0, SEEK_END);
    const long sz = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    if (sz < 0) {
        std::fclose(f);
        return AG2_E_IO;
    }
    *size = (size_t)sz;
    int rc = AG2_OK;
    if (small) {
        small->resize(std::min<size_t>(*size, 512));
        if (std::fread(small->data(), 1, small->size(), f) != small->size()) rc = AG2_E_IO;
    } else {
        rc = ensure_io(c, *size, *size, 64);
        if (!rc && *size && std::fread(c->io_host, 1, *size, f) != *size) rc = AG2_E_IO;
        *pinned = c->io_host;
    }
    std::fclose(f);
    return rc;
}

}  // namespace

int io_reset_tags(Ctx *c, size_t n)
{
    AG2_LAUNCH(c, k_tags_reset, grid_for(n, kIoBlock), kIoBlock, 0, (int64_t)n, c->tag_id, c->tag_gp, c->tag_sfr);
    return AG2_OK;
}

void io_release(Ctx *c)
{
    io_join(c);
    if (c->io_dev) cudaFree(c->io_dev);
    if (c->io_host) cudaFreeHost(c->io_host);
    if (c->io_scratch) cudaFree(c->io_scratch);
    if (c->io_len_dev) cudaFree(c->io_len_dev);
    if (c->io_len_host) cudaFreeHost(c->io_len_host);
    if (c->io_event) cudaEventDestroy(c->io_event);
    if (c->io_stream) cudaStreamDestroy(c->io_stream);
    if (c->tag_id) cudaFree(c->tag_id);
    if (c->tag_gp) cudaFree(c->tag_gp);
    if (c->tag_sfr) cudaFree(c->tag_sfr);
}

}  // namespace ag2

using namespace ag2;

extern "C" {

int ag2_set_tags(ag2_ctx *c, const uint32_t *id, const uint8_t *gp, const double *sfr, int dev)
{
    if (!c) return AG2_E_INVALID;
    if (!c->n) return AG2_OK;
    const cudaMemcpyKind k = dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    if (id) AG2_CUDA(c, cudaMemcpyAsync(c->tag_id, id, c->n * 4, k, c->stream));
    if (gp) AG2_CUDA(c, cudaMemcpyAsync(c->tag_gp, gp, c->n, k, c->stream));
    if (sfr) AG2_CUDA(c, cudaMemcpyAsync(c->tag_sfr, sfr, c->n * 8, k, c->stream));
    if (!dev) AG2_CUDA(c, cudaStreamSynchronize(c->stream));
    return AG2_OK;
}

int ag2_get_tags(ag2_ctx *c, uint32_t *id, uint8_t *gp, double *sfr, int dev)
{
    if (!c) return AG2_E_INVALID;
    if (!c->n) return AG2_OK;
    const cudaMemcpyKind k = dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    if (id) AG2_CUDA(c, cudaMemcpyAsync(id, c->tag_id, c->n * 4, k, c->stream));
    if (gp) AG2_CUDA(c, cudaMemcpyAsync(gp, c->tag_gp, c->n, k, c->stream));
    if (sfr) AG2_CUDA(c, cudaMemcpyAsync(sfr, c->tag_sfr, c->n * 8, k, c->stream));
    if (!dev) AG2_CUDA(c, cudaStreamSynchronize(c->stream));
    return AG2_OK;
}

int ag2_snapshot_size(ag2_ctx *c, int fmt, int64_t count, size_t *bytes)
{
    if (!c || !bytes) return AG2_E_INVALID;
    int rc = check_snapshot_args(c, fmt, count);
    if (rc) return rc;
    *bytes = snapshot_bound(fmt, count);
    return AG2_OK;
}

int ag2_snapshot_encode(ag2_ctx *c, int fmt, int64_t count, double dt, double end_time, double t, void *dst,
                        size_t dst_cap, size_t *len)
{
    if (!c || !dst || !len) return AG2_E_INVALID;
    int rc = check_snapshot_args(c, fmt, count);
    if (rc) return rc;
    io_join(c);
    phase_reset(c);
    if ((rc = encode_snapshot(c, fmt, count, dt, end_time, t))) return rc;
    phase_mark(c, "snapshot encode");
    size_t L = snapshot_bound(fmt, count);
    if (fmt == AG2_FMT_GADGET) {
        AG2_CUDA(c, cudaMemcpyAsync(c->io_len_host, c->io_len_dev, 8, cudaMemcpyDeviceToHost, c->stream));
        AG2_CUDA(c, cudaStreamSynchronize(c->stream));
        L = (size_t)*c->io_len_host;
    }
    *len = L;
    if (L > dst_cap) return set_err(c, AG2_E_INVALID, "destination smaller than the snapshot");
    AG2_CUDA(c, cudaMemcpyAsync(dst, c->io_dev, L, cudaMemcpyDeviceToHost, c->stream));
    phase_mark(c, "snapshot copy");
    AG2_CUDA(c, cudaStreamSynchronize(c->stream));
    phase_finish(c);
    return AG2_OK;
}

int ag2_snapshot_write(ag2_ctx *c, int fmt, int64_t count, double dt, double end_time, double t, const char *path,
                       int async)
{
    if (!c || !path) return AG2_E_INVALID;
    int rc = check_snapshot_args(c, fmt, count);
    if (rc) return rc;
    io_join(c);
    if (c->io_status) {  // an earlier asynchronous write failed and was not collected
        rc = c->io_status;
        c->io_status = 0;
        return set_err(c, rc, c->io_err);
    }
    if ((rc = encode_snapshot(c, fmt, count, dt, end_time, t))) return rc;
    const size_t bound = snapshot_bound(fmt, count);
    if ((rc = ensure_io(c, bound, bound, 0))) return rc;
    AG2_CUDA(c, cudaEventRecord(c->io_event, c->stream));
    AG2_CUDA(c, cudaStreamWaitEvent(c->io_stream, c->io_event, 0));
    AG2_CUDA(c, cudaMemcpyAsync(c->io_host, c->io_dev, bound, cudaMemcpyDeviceToHost, c->io_stream));
    if (fmt == AG2_FMT_GADGET)
        AG2_CUDA(c, cudaMemcpyAsync(c->io_len_host, c->io_len_dev, 8, cudaMemcpyDeviceToHost, c->io_stream));
    AG2_CUDA(c, cudaEventRecord(c->io_event, c->io_stream));
    const bool gadget = fmt == AG2_FMT_GADGET;
    std::string file(path);
    c->io_thread = std::thread([c, gadget, bound, file]() {
        cudaSetDevice(c->device);
        if (cudaEventSynchronize(c->io_event) != cudaSuccess) {
            c->io_status = AG2_E_CUDA;
            c->io_err = "snapshot copy failed";
            return;
        }
        const size_t L = gadget ? (size_t)*c->io_len_host : bound;
        FILE *f = std::fopen(file.c_str(), "wb");
        bool ok = f && (L == 0 || std::fwrite(c->io_host, 1, L, f) == L);
        if (f && std::fclose(f) != 0) ok = false;
        if (!ok) {
            c->io_status = AG2_E_IO;
            c->io_err = "cannot write snapshot file " + file;
        }
    });
    if (!async) return ag2_snapshot_wait(c);
    return AG2_OK;
}

int ag2_snapshot_wait(ag2_ctx *c)
{
    if (!c) return AG2_E_INVALID;
    io_join(c);
    const int s = c->io_status;
    c->io_status = 0;
    if (s) return set_err(c, s, c->io_err);
    return AG2_OK;
}

int ag2_ic_count(const char *path, int fmt, int64_t *n)
{
    if (!path || !n) return AG2_E_INVALID;
    std::vector<uint8_t> head;
    size_t size = 0;
    if (read_file(path, &head, nullptr, &size, nullptr)) return AG2_E_IO;
    if (fmt == AG2_FMT_AG || fmt == AG2_FMT_AGC || fmt == AG2_FMT_AGE) {
        if (size < (size_t)kHdr) return AG2_E_FORMAT;
        const int32_t a = rd_i32(head.data(), 0), b = rd_i32(head.data(), 4), d = rd_i32(head.data(), 8);
        if (a < 0 || b < 0 || d < 0) return AG2_E_FORMAT;
        *n = (int64_t)a + b + d;
        return AG2_OK;
    }
    const size_t off = fmt == AG2_FMT_GADGET ? 4 : fmt == AG2_FMT_MAKEGAL ? 20 : 0;
    if (!off) return AG2_E_FORMAT;
    if (size < off + 24) return AG2_E_FORMAT;
    int64_t s = 0;
    for (int k = 0; k < 6; k++) {
        if (fmt == AG2_FMT_GADGET) s += rd_u32(head.data(), off + 4 * k);
        else {
            const int32_t v = rd_i32(head.data(), off + 4 * k);
            if (v < 0) return AG2_E_FORMAT;
            s += v;
        }
    }
    *n = s;
    return AG2_OK;
}

int ag2_load_ics(ag2_ctx *c, const char *path, int fmt, double *times3)
{
    if (!c || !path) return AG2_E_INVALID;
    if (c->capturing) return set_err(c, AG2_E_INVALID, "load during a stream capture");
    io_join(c);
    uint8_t *img = nullptr;
    size_t size = 0;
    int rc = read_file(path, nullptr, &img, &size, c);
    if (rc == AG2_E_IO) return set_err(c, AG2_E_IO, std::string("cannot read ") + path);
    if (rc) return rc;
    Parsed P;
    std::string why;
    if ((rc = parse_ics(img, size, fmt, P, why))) return set_err(c, rc, why);
    if ((size_t)P.n > c->cap) return set_err(c, AG2_E_CAPACITY, "more particles than the context capacity");
    if (times3)
        for (int k = 0; k < 3; k++) times3[k] = P.times[k];
    const int64_t n = P.n;
    if (n == 0) {
        c->n = 0;
        c->have_tree = false;
        return AG2_OK;
    }
    phase_reset(c);
    AG2_CUDA(c, cudaMemcpyAsync(c->io_dev, img, size, cudaMemcpyHostToDevice, c->stream));
    phase_mark(c, "ic copy");
    Particles &spare = c->st[1];
    IcOut out{c->staging, c->staging + 3 * n, spare.m, spare.U, spare.T, spare.P, spare.vdens,
              c->staging_u8, c->tag_id, c->tag_gp, c->tag_sfr};
    const unsigned g = grid_for(n, kIoBlock);
    const bool has_vel = fmt == AG2_FMT_AGE || fmt == AG2_FMT_GADGET || fmt == AG2_FMT_MAKEGAL;
    const bool has_u = has_vel;
    if (fmt == AG2_FMT_AG) AG2_LAUNCH(c, k_ic_records<AG2_FMT_AG>, g, kIoBlock, 0, n, c->io_dev, out);
    else if (fmt == AG2_FMT_AGC) AG2_LAUNCH(c, k_ic_records<AG2_FMT_AGC>, g, kIoBlock, 0, n, c->io_dev, out);
    else if (fmt == AG2_FMT_AGE) AG2_LAUNCH(c, k_ic_records<AG2_FMT_AGE>, g, kIoBlock, 0, n, c->io_dev, out);
    else AG2_LAUNCH(c, k_ic_gadget, g, kIoBlock, 0, P.g, c->io_dev, out);
    rc = upload_common(c, (size_t)n, c->staging, has_vel ? c->staging + 3 * n : nullptr, spare.m,
                       has_u ? spare.U : nullptr, c->staging_u8);
    if (rc) return rc;
    if (fmt == AG2_FMT_AG || fmt == AG2_FMT_AGC || fmt == AG2_FMT_AGE)
        AG2_LAUNCH(c, k_ic_fields, g, kIoBlock, 0, n, spare.T, fmt == AG2_FMT_AGE ? spare.P : nullptr, spare.vdens,
                   c->S());
    phase_mark(c, "ic decode");
    AG2_CUDA(c, cudaStreamSynchronize(c->stream));
    phase_finish(c);
    return AG2_OK;
}

}  // extern "C"
