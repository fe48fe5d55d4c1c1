// ag2_api.cu -- the C-ABI of include/ag2.h: context, particle upload and
// download in the caller's order, the step driver and tree introspection.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "ag2_internal.cuh"

namespace ag2 {

int run_close_step(Ctx *c, double dt, double f);

int set_err(Ctx *c, int code, const std::string &msg)
{
    if (c) c->err = msg;
    return code;
}

int cuda_check(Ctx *c, cudaError_t e, const char *what)
{
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    return set_err(c, e == cudaErrorMemoryAllocation ? AG2_E_NOMEM : AG2_E_CUDA, m);
}

void phase_reset(Ctx *c)
{
    if (!c->timing) return;
    c->nphase = 0;
    cudaEventRecord(c->ev[0], c->stream);
}

void phase_mark(Ctx *c, const char *name)
{
    if (!c->timing || c->nphase >= Ctx::kMaxPhases) return;
    c->phase_name[c->nphase] = name;
    cudaEventRecord(c->ev[c->nphase + 1], c->stream);
    c->nphase++;
}

void phase_finish(Ctx *c)
{
    if (!c->timing || c->nphase == 0) return;
    cudaEventSynchronize(c->ev[c->nphase]);
    for (int k = 0; k < c->nphase; k++) {
        float ms = 0;
        cudaEventElapsedTime(&ms, c->ev[k], c->ev[k + 1]);
        c->phase_ms[k] = ms;
    }
    c->phase_count = c->nphase;
}

int sync_ctl(Ctx *c)
{
    AG2_CUDA(c, cudaMemcpyAsync(c->ctl_host, c->ctl, sizeof(Ctx::Ctl), cudaMemcpyDeviceToHost, c->stream));
    AG2_CUDA(c, cudaStreamSynchronize(c->stream));
    return AG2_OK;
}

namespace {

constexpr int kBlock = 256;

// Caller's arrays (upload order) into the state.  With `prev`, slot t takes
// upload index prev[t], the particle it held before: the same particle set
// uploaded again keeps the last build's spatial order, so the next build moves
// neighbours together instead of starting from the caller's order.  (A gather:
// scattered reads of the caller's records, whole-sector writes of the state.)
__global__ void k_unpack(int n, const double *pos, const double *vel, const double *mass, const double *U,
                         const uint8_t *type, const int32_t *prev, Particles s, Ctx::Ctl *ctl)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int i = prev ? prev[t] : t;
    double x = pos[3 * (size_t)i], y = pos[3 * (size_t)i + 1], z = pos[3 * (size_t)i + 2];
    if (!isfinite(x) || !isfinite(y) || !isfinite(z)) atomicExch(&ctl->err_code, (int)AG2_E_NAN);
    s.px[t] = x;
    s.py[t] = y;
    s.pz[t] = z;
    s.vx[t] = vel ? vel[3 * (size_t)i] : 0.0;
    s.vy[t] = vel ? vel[3 * (size_t)i + 1] : 0.0;
    s.vz[t] = vel ? vel[3 * (size_t)i + 2] : 0.0;
    s.ax[t] = s.ay[t] = s.az[t] = 0.0;
    s.m[t] = mass[i];
    s.U[t] = U ? U[i] : 0.0;
    s.dUdt[t] = 0.0;
    s.h[t] = s.rho[t] = s.P[t] = s.T[t] = s.vdens[t] = 0.0;
    s.tstep[t] = s.tnext[t] = 0.0;
    s.type[t] = type[i];
    s.id[t] = i;
}

// The state back into upload order (slot i holds upload index i): a scatter by
// each slot's upload index, for an instance layout the current permutation
// does not keep apart.
__global__ void k_to_upload_order(int n, Particles s, Particles d)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int i = s.id[t];
    d.px[i] = s.px[t];
    d.py[i] = s.py[t];
    d.pz[i] = s.pz[t];
    d.vx[i] = s.vx[t];
    d.vy[i] = s.vy[t];
    d.vz[i] = s.vz[t];
    d.ax[i] = s.ax[t];
    d.ay[i] = s.ay[t];
    d.az[i] = s.az[t];
    d.m[i] = s.m[t];
    d.U[i] = s.U[t];
    d.dUdt[i] = s.dUdt[t];
    d.h[i] = s.h[t];
    d.rho[i] = s.rho[t];
    d.P[i] = s.P[t];
    d.T[i] = s.T[t];
    d.vdens[i] = s.vdens[t];
    d.tstep[i] = s.tstep[t];
    d.tnext[i] = s.tnext[t];
    d.type[i] = s.type[t];
    d.id[i] = i;
}

__device__ double *field1(Particles &s, int f)
{
    switch (f) {
    case AG2_MASS: return s.m;
    case AG2_H: return s.h;
    case AG2_RHO: return s.rho;
    case AG2_P: return s.P;
    case AG2_T: return s.T;
    case AG2_U: return s.U;
    case AG2_DUDT: return s.dUdt;
    case AG2_VDENS: return s.vdens;
    case AG2_TSTEP: return s.tstep;
    case AG2_TNEXT: return s.tnext;
    }
    return nullptr;
}

__device__ void field3(Particles &s, int f, double *&x, double *&y, double *&z)
{
    if (f == AG2_POS) { x = s.px; y = s.py; z = s.pz; }
    else if (f == AG2_VEL) { x = s.vx; y = s.vy; z = s.vz; }
    else { x = s.ax; y = s.ay; z = s.az; }
}

// tree order -> caller order
__global__ void k_gather_out(int n, Particles s, int f, double *out)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int o = s.id[i];
    if (f <= AG2_ACC) {
        double *x, *y, *z;
        field3(s, f, x, y, z);
        out[3 * o] = x[i];
        out[3 * o + 1] = y[i];
        out[3 * o + 2] = z[i];
    } else {
        out[o] = field1(s, f)[i];
    }
}

// caller order -> tree order
__global__ void k_scatter_in(int n, Particles s, int f, const double *in)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int o = s.id[i];
    if (f <= AG2_ACC) {
        double *x, *y, *z;
        field3(s, f, x, y, z);
        x[i] = in[3 * o];
        y[i] = in[3 * o + 1];
        z[i] = in[3 * o + 2];
    } else {
        field1(s, f)[i] = in[o];
    }
}

int alloc_particles(Ctx *c, Particles &p, size_t cap)
{
    double **d[] = {&p.px, &p.py, &p.pz, &p.vx, &p.vy, &p.vz, &p.ax, &p.ay, &p.az, &p.m,
                    &p.U,  &p.dUdt, &p.h, &p.rho, &p.P, &p.T, &p.vdens, &p.tstep, &p.tnext};
    for (double **q : d)
        if (cudaMalloc(q, cap * sizeof(double)) != cudaSuccess)
            return set_err(c, AG2_E_NOMEM, "particle allocation failed");
    if (cudaMalloc(&p.type, cap) != cudaSuccess || cudaMalloc(&p.id, cap * sizeof(int32_t)) != cudaSuccess)
        return set_err(c, AG2_E_NOMEM, "particle allocation failed");
    return AG2_OK;
}

void free_particles(Particles &p)
{
    double *d[] = {p.px, p.py, p.pz, p.vx, p.vy, p.vz, p.ax, p.ay, p.az, p.m, p.U, p.dUdt, p.h, p.rho, p.P, p.T,
                   p.vdens, p.tstep, p.tnext};
    for (double *q : d) cudaFree(q);
    cudaFree(p.type);
    cudaFree(p.id);
    p = Particles{};
}

void free_nodes(Nodes &d)
{
    void *ps[] = {d.start, d.count, d.ndrop, d.first, d.parent, d.leafpos, d.level, d.mode, d.needs,
                  d.cx,    d.cy,    d.cz,    d.bkey,  d.mom,   d.tsum,
                  d.wrec, d.flag, d.rho,
                  d.radius, d.inst, d.nlx, d.lint, d.lil};
    for (void *q : ps) cudaFree(q);
    d = Nodes{};
}

bool valid_params(const ag2_params *p)
{
    return p && p->split_threshold >= 1 && (p->precision == AG2_PREC_FP64 || p->precision == AG2_PREC_FP32) &&
           p->theta > 0.0 && p->group_size >= 0 && p->group_size <= 32;
}

__global__ void k_pinst(const int64_t *first, int32_t *pinst)
{
    const int k = blockIdx.x;
    for (int64_t i = first[k] + threadIdx.x; i < first[k + 1]; i += blockDim.x) pinst[i] = k;
}

template <class T>
bool realloc_dev(T *&p, size_t n)
{
    if (p) cudaFree(p);
    p = nullptr;
    return cudaMalloc((void **)&p, (n ? n : 1) * sizeof(T)) == cudaSuccess;
}

}  // namespace

// particles per walk group (0 reads as 32)
int group_size_of(const ag2_params &p) { return p.group_size > 0 ? p.group_size : 32; }

// Walk groups of the current instance layout: runs of group_size consecutive
// slots that never straddle two instances.  They depend on the layout and the
// group size only, so a new table is valid for the tree already built.
int build_groups(Ctx *c)
{
    const int gs = group_size_of(c->prm);
    std::vector<int4> g;
    for (int k = 0; k < c->n_inst; k++) {
        const int64_t b = c->inst_first_h[k], e = c->inst_first_h[k + 1];
        for (int64_t s = b; s < e; s += gs) g.push_back(make_int4((int)s, (int)std::min<int64_t>(gs, e - s), k, 0));
    }
    if (g.size() > c->groups_cap) {
        if (!realloc_dev(c->groups, g.size()) || !realloc_dev(c->retry_groups, g.size()))
            return set_err(c, AG2_E_NOMEM, "group table allocation failed");
        c->groups_cap = g.size();
    }
    if (!g.empty())
        AG2_CUDA(c, cudaMemcpyAsync(c->groups, g.data(), g.size() * sizeof(int4), cudaMemcpyHostToDevice, c->stream));
    AG2_CUDA(c, cudaStreamSynchronize(c->stream));  // g goes out of scope
    c->ngroups = (int32_t)g.size();
    c->groups_gs = gs;
    return AG2_OK;
}


int upload_common(Ctx *c, size_t n, const double *pos, const double *vel, const double *mass, const double *U,
                  const uint8_t *type)
{
    AG2_CUDA(c, cudaMemsetAsync(&c->ctl->err_code, 0, sizeof(int32_t), c->stream));
    // the same count again: keep the slots of the last build (each slot reads
    // and rewrites only its own id, so the current buffer may be the target)
    const int32_t *prev = (c->n == n && !c->upload_order) ? c->S().id : nullptr;
    c->cur = 0;
    AG2_LAUNCH(c, k_unpack, grid_for(n, kBlock), kBlock, 0, (int)n, pos, vel, mass, U, type, prev, c->S(), c->ctl);
    if (!prev) c->upload_order = true;
    c->n = n;
    c->have_tree = false;
    c->gas_stats_dirty = true;
    c->n_inst = 1;
    c->inst_dirty = true;
    c->inst_explicit = false;
    c->graph_epoch++;
    int rc = sync_ctl(c);
    if (rc) return rc;
    if (c->ctl_host->err_code == AG2_E_NAN) return set_err(c, AG2_E_NAN, "non-finite particle position");
    return AG2_OK;
}

// Upload the instance tables and walk groups when the instance layout changed.
int ensure_instance_tables(Ctx *c)
{
    if (!c->inst_dirty) return AG2_OK;
    const int K = c->n_inst;
    if (!c->upload_order && K > 1 && c->inst_first_h != c->perm_first) {
        // the slots hold a permutation made under another layout: instance k
        // must own slots [first[k], first[k+1]) again
        AG2_LAUNCH(c, k_to_upload_order, grid_for(c->n, kBlock), kBlock, 0, (int)c->n, c->S(), c->st[c->cur ^ 1]);
        c->cur ^= 1;
        c->upload_order = true;
    }
    if ((size_t)K > c->inst_cap) {
        bool ok = realloc_dev(c->inst_first, K + 1) && realloc_dev(c->inst_R, K) && realloc_dev(c->inst_massInH, K) &&
                  realloc_dev(c->gas_off, K) && realloc_dev(c->gas_uni, K) && realloc_dev(c->gas_cnt, K) &&
                  realloc_dev(c->gas_kmin, K) && realloc_dev(c->gas_kmax, K) && realloc_dev(c->width_thr, K) &&
                  realloc_dev(c->wsum_final, K);
        if (!ok) return set_err(c, AG2_E_NOMEM, "instance table allocation failed");
        c->inst_cap = K;
    }
    if (K == 1 && !c->inst_explicit) {
        c->inst_first_h = {0, (int64_t)c->n};
        c->inst_massInH_h = {c->prm.massInH};
    }
    AG2_CUDA(c, cudaMemcpyAsync(c->inst_massInH, c->inst_massInH_h.data(), K * sizeof(double), cudaMemcpyHostToDevice,
                                c->stream));
    if (c->inst_first_h == c->inst_tab_first) {  // same layout (an upload of the same particles): tables stand
        if (c->groups_gs != group_size_of(c->prm)) {
            int rc = build_groups(c);
            if (rc) return rc;
        }
        c->inst_dirty = false;
        c->gas_stats_dirty = true;
        return AG2_OK;
    }
    AG2_CUDA(c, cudaMemcpyAsync(c->inst_first, c->inst_first_h.data(), (K + 1) * sizeof(int64_t),
                                cudaMemcpyHostToDevice, c->stream));
    // root-width summation tasks (ag2_build.cu): one sequential task per instance
    // up to 4096 particles, a 64-ary tree of sequential runs above
    {
        std::vector<std::vector<int4>> lv(1);
        std::vector<int32_t> fin(K);
        int32_t nbuf = 0;
        // level 0 tasks read particles; a task's z is its destination pair
        std::vector<std::pair<int32_t, int32_t>> cur(K);  // per instance: (first pair, count) of its current level
        for (int k = 0; k < K; k++) {
            const int64_t b = c->inst_first_h[k], n = c->inst_first_h[k + 1] - b;
            const int64_t run = n <= kSeqWidthMax ? std::max<int64_t>(n, 1) : kWsumRun;
            const int32_t cnt = (int32_t)((n + run - 1) / run);
            cur[k] = {nbuf, std::max(cnt, 1)};
            for (int64_t j = 0; j < std::max<int64_t>(n, 1); j += run)
                lv[0].push_back(make_int4((int)(b + j), (int)std::min(run, n - j), nbuf++, k));
            if (n == 0) {
                lv[0].back().y = 0;
            }
        }
        for (;;) {
            std::vector<int4> next;
            bool any = false;
            for (int k = 0; k < K; k++) {
                auto [p0, cnt] = cur[k];
                if (cnt <= 1) {
                    fin[k] = p0;
                    continue;
                }
                any = true;
                const int32_t nn = (cnt + 63) / 64;
                const int32_t q0 = nbuf;
                for (int32_t j = 0; j < cnt; j += 64) next.push_back(make_int4(p0 + j, std::min(64, cnt - j), nbuf++, k));
                cur[k] = {q0, nn};
            }
            if (!any) break;
            lv.push_back(std::move(next));
        }
        std::vector<int4> all;
        c->wsum_level.assign(1, 0);
        for (auto &l : lv) {
            all.insert(all.end(), l.begin(), l.end());
            c->wsum_level.push_back((int32_t)all.size());
        }
        if (!realloc_dev(c->wsum_task, all.size()) || !realloc_dev(c->width_part, 2 * (size_t)std::max(nbuf, 1)))
            return set_err(c, AG2_E_NOMEM, "root width table allocation failed");
        AG2_CUDA(c, cudaMemcpyAsync(c->wsum_task, all.data(), all.size() * sizeof(int4), cudaMemcpyHostToDevice,
                                    c->stream));
        AG2_CUDA(c, cudaMemcpyAsync(c->wsum_final, fin.data(), K * sizeof(int32_t), cudaMemcpyHostToDevice,
                                    c->stream));
        // the long sequential sums, which the particle-level kernel leaves to k_wsum_long
        std::vector<int32_t> longt;
        for (int32_t t = 0; t < c->wsum_level[1]; t++)
            if (all[t].y > kWsumRun) longt.push_back(t);
        c->nwsum_long = (int32_t)longt.size();
        if (!longt.empty()) {
            if (!realloc_dev(c->wsum_long, longt.size()))
                return set_err(c, AG2_E_NOMEM, "root width table allocation failed");
            AG2_CUDA(c, cudaMemcpyAsync(c->wsum_long, longt.data(), longt.size() * sizeof(int32_t),
                                        cudaMemcpyHostToDevice, c->stream));
        }
        AG2_CUDA(c, cudaStreamSynchronize(c->stream));
    }
    {
        int rc = build_groups(c);
        if (rc) return rc;
    }
    if (c->n) AG2_LAUNCH(c, k_pinst, K, 256, 0, c->inst_first, c->pinst);
    AG2_CUDA(c, cudaStreamSynchronize(c->stream));  // host vectors above go out of scope
    c->inst_tab_first = c->inst_first_h;
    c->inst_dirty = false;
    c->gas_stats_dirty = true;
    return AG2_OK;
}

}  // namespace ag2

using namespace ag2;


extern "C" {

void ag2_default_params(ag2_params *p)
{
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->G = 1.0;
    p->e0 = 0.01;
    p->theta = 0.5;
    p->massInH = 0.0;
    p->split_threshold = 100;
    p->precision = AG2_PREC_FP32;
    p->group_size = 32;
}

int ag2_create(ag2_ctx **out, const ag2_params *params, size_t capacity)
{
    if (!out) return AG2_E_INVALID;
    *out = nullptr;
    if (!valid_params(params) || capacity > (size_t)INT32_MAX / 4) return AG2_E_INVALID;
    ag2_ctx *c = new (std::nothrow) ag2_ctx();
    if (!c) return AG2_E_NOMEM;
    c->prm = *params;
    cudaGetDevice(&c->device);
    cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, c->device);
    if (const char *dbg = std::getenv("AG2_DEBUG_SYNC")) c->debug_sync = dbg[0] == '1';
    size_t cap = std::max(capacity, (size_t)1);
    c->cap = cap;
    int rc = AG2_OK;
    cudaError_t e = cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        rc = cuda_check(c, e, "cudaStreamCreate");
        delete c;
        return rc;
    }
    c->stream = c->own_stream;
    bool ok = alloc_particles(c, c->st[0], cap) == AG2_OK && alloc_particles(c, c->st[1], cap) == AG2_OK;
    ok = ok && cudaMalloc(&c->perm, cap * 4) == cudaSuccess && cudaMalloc(&c->perm2, cap * 4) == cudaSuccess &&
         cudaMalloc(&c->posnode, cap * 4) == cudaSuccess && cudaMalloc(&c->posnode2, cap * 4) == cudaSuccess &&
         cudaMalloc(&c->pnode, cap * 4) == cudaSuccess && cudaMalloc(&c->refnode, cap * 4) == cudaSuccess && cudaMalloc(&c->slot_of, cap * 4) == cudaSuccess && cudaMalloc(&c->rdist, cap * sizeof(double2)) == cudaSuccess && cudaMalloc(&c->finalnode, cap * 4) == cudaSuccess &&
         cudaMalloc(&c->nodelist, cap * 4) == cudaSuccess && cudaMalloc(&c->gas_slots, cap * 4) == cudaSuccess && cudaMalloc(&c->drop_list, 65536 * 4) == cudaSuccess && cudaMalloc(&c->digit, 2 * cap) == cudaSuccess &&
         cudaMalloc(&c->staging, 6 * cap * sizeof(double)) == cudaSuccess &&
         cudaMalloc(&c->staging_u8, cap) == cudaSuccess &&
         cudaMalloc(&c->pinst, cap * 4) == cudaSuccess &&
         cudaMalloc(&c->perm_final, cap * 4) == cudaSuccess && cudaMalloc(&c->ap[0], cap * 4) == cudaSuccess &&
         cudaMalloc(&c->ap[1], cap * 4) == cudaSuccess && cudaMalloc(&c->nl[0], cap * 4) == cudaSuccess &&
         cudaMalloc(&c->nl[1], cap * 4) == cudaSuccess &&
         cudaMalloc(&c->lroots, cap * 4) == cudaSuccess &&
         cudaMalloc(&c->pkey, 6 * cap * sizeof(int64_t)) == cudaSuccess &&
         cudaMalloc(&c->tag_id, cap * 4) == cudaSuccess && cudaMalloc(&c->tag_gp, cap) == cudaSuccess &&
         cudaMalloc(&c->tag_sfr, cap * sizeof(double)) == cudaSuccess &&
         cudaMalloc(&c->ctl, sizeof(Ctx::Ctl)) == cudaSuccess &&
         cudaMallocHost(&c->ctl_host, sizeof(Ctx::Ctl)) == cudaSuccess;
    if (ok) ok = ensure_node_capacity(c, 4 * cap + 1024) == AG2_OK;
    if (!ok) {
        ag2_destroy(c);
        return AG2_E_NOMEM;
    }
    cudaMemsetAsync(c->ctl, 0, sizeof(Ctx::Ctl), c->stream);
    std::memset(c->ctl_host, 0, sizeof(Ctx::Ctl));
    cudaStreamSynchronize(c->stream);
    *out = c;
    return AG2_OK;
}

int ag2_destroy(ag2_ctx *c)
{
    if (!c) return AG2_E_INVALID;
    if (c->stream) cudaStreamSynchronize(c->stream);
    io_release(c);
    free_particles(c->st[0]);
    free_particles(c->st[1]);
    free_nodes(c->nd);
    void *ps[] = {c->perm, c->perm2, c->posnode, c->posnode2, c->pnode, c->refnode, c->slot_of, c->rdist, c->finalnode,
                  c->nodelist, c->gas_slots, c->drop_list, c->digit, c->hist, c->cursor, c->gas_prefix, c->staging, c->staging_u8,
                  c->width_part, c->width_thr, c->wsum_task, c->wsum_final, c->wsum_long, c->ctl, c->pinst, c->groups, c->retry_groups, c->inst_first, c->inst_R,
                  c->inst_massInH, c->gas_off, c->gas_uni, c->gas_cnt, c->gas_kmin, c->gas_kmax,
                  c->perm_final, c->ap[0], c->ap[1], c->nl[0], c->nl[1], c->pkey, c->lroots};
    for (void *q : ps) cudaFree(q);
    if (c->ctl_host) cudaFreeHost(c->ctl_host);
    if (c->gas_pin) cudaFreeHost(c->gas_pin);
    if (c->ctl_snap) cudaFreeHost(c->ctl_snap);
    for (auto &e : c->snap_ev)
        if (e) cudaEventDestroy(e);
    if (c->inst_R_pin) cudaFreeHost(c->inst_R_pin);
    if (c->inst_R_rb) cudaFreeHost(c->inst_R_rb);
    for (auto &x : c->step_exec)
        if (x) cudaGraphExecDestroy(x);
    if (c->side_stream) cudaStreamDestroy(c->side_stream);
    if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
    for (int b = 0; b < 2; b++) {
        if (c->dl_gathered[b]) cudaEventDestroy(c->dl_gathered[b]);
        if (c->dl_copied[b]) cudaEventDestroy(c->dl_copied[b]);
        if (c->up_ev[b]) cudaEventDestroy(c->up_ev[b]);
    }
    if (c->acc_stage) cudaFree(c->acc_stage);
    if (c->blk_key) cudaFree(c->blk_key);
    for (auto &e : c->ev)
        if (e) cudaEventDestroy(e);
    if (c->own_stream) cudaStreamDestroy(c->own_stream);
    delete c;
    return AG2_OK;
}

int ag2_set_params(ag2_ctx *c, const ag2_params *p)
{
    if (!c || !valid_params(p)) return set_err(c, AG2_E_INVALID, "invalid parameters");
    bool retree = p->split_threshold != c->prm.split_threshold;
    const bool regroup = group_size_of(*p) != group_size_of(c->prm);
    c->prm = *p;
    if (retree) c->have_tree = false;
    if (regroup) {
        // the groups depend on the layout and the group size only: a built
        // layout gets its new table now (valid for the tree already built)
        if (!c->inst_dirty && !c->inst_tab_first.empty()) {
            int rc = build_groups(c);
            if (rc) return rc;
        }
    }
    if (c->n_inst == 1 && !c->inst_explicit) c->inst_massInH_h = {p->massInH};
    c->graph_epoch++;
    return AG2_OK;
}

int ag2_get_params(const ag2_ctx *c, ag2_params *p)
{
    if (!c || !p) return AG2_E_INVALID;
    *p = c->prm;
    return AG2_OK;
}

int ag2_set_stream(ag2_ctx *c, void *stream)
{
    if (!c) return AG2_E_INVALID;
    c->stream = stream ? (cudaStream_t)stream : c->own_stream;
    c->graph_epoch++;
    return AG2_OK;
}

const char *ag2_last_error_string(const ag2_ctx *c) { return c ? c->err.c_str() : "no context"; }

int ag2_upload(ag2_ctx *c, size_t n, const double *pos, const double *vel, const double *mass, const double *U,
               const uint8_t *type)
{
    if (!c) return AG2_E_INVALID;
    if (n > c->cap) return set_err(c, AG2_E_CAPACITY, "more particles than the context capacity");
    if (n && (!pos || !mass || !type)) return set_err(c, AG2_E_INVALID, "pos, mass and type are required");
    if (n == 0) {
        c->n = 0;
        c->have_tree = false;
        return AG2_OK;
    }
    // host -> staging (positions | velocities), masses and U into the spare
    // state half, which the unpack kernel does not write
    Particles &spare = c->st[1];
    double *pos_d = c->staging, *vel_d = vel ? c->staging + 3 * n : nullptr;
    AG2_CUDA(c, cudaMemcpyAsync(pos_d, pos, 3 * n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    if (vel) AG2_CUDA(c, cudaMemcpyAsync(vel_d, vel, 3 * n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    AG2_CUDA(c, cudaMemcpyAsync(spare.m, mass, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    if (U) AG2_CUDA(c, cudaMemcpyAsync(spare.U, U, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    AG2_CUDA(c, cudaMemcpyAsync(c->staging_u8, type, n, cudaMemcpyHostToDevice, c->stream));
    int rc = upload_common(c, n, pos_d, vel_d, spare.m, U ? spare.U : nullptr, c->staging_u8);
    return rc ? rc : io_reset_tags(c, n);
}

int ag2_upload_device(ag2_ctx *c, size_t n, const double *pos, const double *vel, const double *mass,
                      const double *U, const uint8_t *type)
{
    if (!c) return AG2_E_INVALID;
    if (n > c->cap) return set_err(c, AG2_E_CAPACITY, "more particles than the context capacity");
    if (n && (!pos || !mass || !type)) return set_err(c, AG2_E_INVALID, "pos, mass and type are required");
    if (n == 0) {
        c->n = 0;
        c->have_tree = false;
        return AG2_OK;
    }
    int rc = upload_common(c, n, pos, vel, mass, U, type);
    return rc ? rc : io_reset_tags(c, n);
}

int ag2_set_field(ag2_ctx *c, int f, const double *src, int src_is_device)
{
    if (!c || !src || f < AG2_POS || f > AG2_TNEXT) return set_err(c, AG2_E_INVALID, "bad field");
    size_t cnt = (f <= AG2_ACC ? 3 : 1) * c->n;
    if (!c->n) return AG2_OK;
    const double *in = src;
    if (!src_is_device) {
        AG2_CUDA(c, cudaMemcpyAsync(c->staging, src, cnt * sizeof(double), cudaMemcpyHostToDevice, c->stream));
        in = c->staging;
    }
    AG2_LAUNCH(c, k_scatter_in, grid_for(c->n, kBlock), kBlock, 0, (int)c->n, c->S(), f, in);
    if (f == AG2_POS || f == AG2_MASS) c->have_tree = false;
    if (f == AG2_MASS) c->gas_stats_dirty = true;
    c->graph_epoch++;
    return AG2_OK;
}

int ag2_download(ag2_ctx *c, int f, double *dst, int dst_is_device)
{
    if (!c || !dst || f < AG2_POS || f > AG2_TNEXT) return set_err(c, AG2_E_INVALID, "bad field");
    size_t cnt = (f <= AG2_ACC ? 3 : 1) * c->n;
    if (!c->n) return AG2_OK;
    double *out = dst_is_device ? dst : c->staging;
    AG2_LAUNCH(c, k_gather_out, grid_for(c->n, kBlock), kBlock, 0, (int)c->n, c->S(), f, out);
    if (!dst_is_device) {
        AG2_CUDA(c, cudaMemcpyAsync(dst, c->staging, cnt * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        AG2_CUDA(c, cudaStreamSynchronize(c->stream));
    }
    return AG2_OK;
}

// Read-back pipeline of ag2_download_fields and ag2_step_host: field k is
// gathered into upload order in staging half k % 2 on the context's stream and
// copied to the host on the copy stream, so the next gather (or other device
// work) overlaps the copy; dl_end waits for every copy.
static int dl_begin(Ctx *c)
{
    if (c->copy_stream) return AG2_OK;
    AG2_CUDA(c, cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
    for (int b = 0; b < 2; b++) {
        AG2_CUDA(c, cudaEventCreateWithFlags(&c->dl_gathered[b], cudaEventDisableTiming));
        AG2_CUDA(c, cudaEventCreateWithFlags(&c->dl_copied[b], cudaEventDisableTiming));
    }
    return AG2_OK;
}
static int dl_field(Ctx *c, int k, int field, double *dst)
{
    const int b = k & 1;
    double *half = c->staging + (size_t)b * 3 * c->n;
    const size_t cnt = (field <= AG2_ACC ? 3 : 1) * c->n;
    if (k >= 2) AG2_CUDA(c, cudaStreamWaitEvent(c->stream, c->dl_copied[b], 0));  // the half is free again
    AG2_LAUNCH(c, k_gather_out, grid_for(c->n, kBlock), kBlock, 0, (int)c->n, c->S(), field, half);
    AG2_CUDA(c, cudaEventRecord(c->dl_gathered[b], c->stream));
    AG2_CUDA(c, cudaStreamWaitEvent(c->copy_stream, c->dl_gathered[b], 0));
    AG2_CUDA(c, cudaMemcpyAsync(dst, half, cnt * sizeof(double), cudaMemcpyDeviceToHost, c->copy_stream));
    AG2_CUDA(c, cudaEventRecord(c->dl_copied[b], c->copy_stream));
    return AG2_OK;
}
static int dl_end(Ctx *c)
{
    AG2_CUDA(c, cudaStreamSynchronize(c->copy_stream));
    return AG2_OK;
}
// Error exit of a call that may have queued read-backs: wait for every copy
// already on the copy stream, so that none still writes into the caller's
// buffers or reads the staging area after the call returns (the next upload
// or download reuses staging on the context's stream).  The first error is
// the one reported.
static int dl_abort(Ctx *c, int rc)
{
    if (c->copy_stream) cudaStreamSynchronize(c->copy_stream);
    return rc;
}

int ag2_download_fields(ag2_ctx *c, int nf, const int *fields, double *const *dst)
{
    if (!c || nf < 0 || (nf && (!fields || !dst))) return AG2_E_INVALID;
    for (int k = 0; k < nf; k++)
        if (!dst[k] || fields[k] < AG2_POS || fields[k] > AG2_TNEXT) return set_err(c, AG2_E_INVALID, "bad field");
    if (!c->n || !nf) return AG2_OK;
    int rc;
    if ((rc = dl_begin(c))) return rc;
    for (int k = 0; k < nf; k++)
        if ((rc = dl_field(c, k, fields[k], dst[k]))) return dl_abort(c, rc);
    return dl_end(c);
}

int ag2_inject_fault(ag2_ctx *c, int site, int code)
{
    if (!c || site < 0 || site > 1 || code > 0) return AG2_E_INVALID;
    c->inject_site = site;
    c->inject_code = code;
    return AG2_OK;
}

size_t ag2_count(const ag2_ctx *c) { return c ? c->n : 0; }

int ag2_build_tree(ag2_ctx *c)
{
    if (!c) return AG2_E_INVALID;
    phase_reset(c);
    int rc = build_tree(c);
    phase_finish(c);
    return rc;
}

int ag2_visual_density(ag2_ctx *c, double R)
{
    if (!c) return AG2_E_INVALID;
    return run_visual_density(c, R);
}

int ag2_sph_density(ag2_ctx *c)
{
    if (!c) return AG2_E_INVALID;
    return run_sph_density(c);
}

static int check_walk(Ctx *c)
{
    int rc = sync_ctl(c);
    if (rc) return rc;
    c->inter_grav = (int64_t)c->ctl_host->inter_grav;
    c->inter_sph = (int64_t)c->ctl_host->inter_sph;
    if (c->ctl_host->err_code == AG2_E_STACK)
        return set_err(c, AG2_E_STACK, "walk stack overflow (tree deeper than the walk stack supports)");
    return AG2_OK;
}

int ag2_forces(ag2_ctx *c)
{
    if (!c) return AG2_E_INVALID;
    AG2_CUDA(c, cudaMemsetAsync(&c->ctl->err_code, 0, sizeof(int32_t), c->stream));
    int rc = run_forces(c);
    if (rc) return rc;
    return check_walk(c);
}

int ag2_kick(ag2_ctx *c, double dt) { return c ? run_kick(c, dt) : AG2_E_INVALID; }
int ag2_drift(ag2_ctx *c, double dt) { return c ? run_drift(c, dt) : AG2_E_INVALID; }
int ag2_kick_drift(ag2_ctx *c, double dt) { return c ? run_kick_drift(c, dt) : AG2_E_INVALID; }
int ag2_ueuler(ag2_ctx *c, double dt) { return c ? run_ueuler(c, dt) : AG2_E_INVALID; }
int ag2_scale_positions(ag2_ctx *c, double f) { return c ? run_scale(c, f) : AG2_E_INVALID; }

// ---- step graphs -------------------------------------------------------------

static unsigned long long fnv(unsigned long long h, const void *p, size_t n)
{
    const unsigned char *b = static_cast<const unsigned char *>(p);
    for (size_t i = 0; i < n; i++) h = (h ^ b[i]) * 1099511628211ull;
    return h;
}

// everything a captured step bakes in: sizes, pointers of every pool, parameters
static unsigned long long step_key(Ctx *c, double dt, double hubble, int with_visual, double Rv)
{
    unsigned long long h = 1469598103934665603ull;
    const void *ptrs[] = {c->nd.start, c->nd.bkey, c->nd.wrec, c->nd.lint, c->hist, c->stream, c->gas_prefix,
                          c->groups, c->inst_first, c->pkey};
    h = fnv(h, ptrs, sizeof(ptrs));
    const int64_t sizes[] = {(int64_t)c->n, c->n_inst, (int64_t)c->node_cap, (int64_t)c->hist_cap, c->ngas,
                             c->walk_variant, c->ngroups, c->groups_gs, with_visual, c->graph_epoch};
    h = fnv(h, sizes, sizeof(sizes));
    h = fnv(h, &c->prm, sizeof(c->prm));
    const double d[] = {dt, hubble, Rv};
    return fnv(h, d, sizeof(d));
}

static int capture_step(Ctx *c, double dt, double hubble, int with_visual, double Rv, cudaGraphExec_t *exec,
                        int64_t *nlaunch)
{
    const int64_t l0 = c->launches;
    const bool had_tree = c->have_tree;
    c->capturing = true;
    cudaError_t e = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal);
    int rc = e == cudaSuccess ? AG2_OK : cuda_check(c, e, "cudaStreamBeginCapture");
    if (!rc) rc = run_kick_drift(c, dt);
    if (!rc) rc = build_tree_captured(c);
    if (!rc && with_visual) rc = run_visual_density(c, Rv);
    if (!rc) rc = run_sph_density(c);
    if (!rc) {
        e = cudaMemsetAsync(&c->ctl->err_code, 0, sizeof(int32_t), c->stream);
        if (e != cudaSuccess) rc = cuda_check(c, e, "cudaMemsetAsync");
    }
    if (!rc) rc = run_forces(c);
    if (!rc) rc = run_close_step(c, dt, hubble);
    if (!rc) {
        e = cudaMemcpyAsync(c->ctl_host, c->ctl, sizeof(Ctx::Ctl), cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(c->inst_R_pin, c->inst_R, c->n_inst * sizeof(double), cudaMemcpyDeviceToHost,
                                c->stream);
        if (e != cudaSuccess) rc = cuda_check(c, e, "cudaMemcpyAsync");
    }
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(c->stream, &g);
    c->capturing = false;
    c->have_tree = had_tree;
    // launches per replay: those outside the two loops; the loop bodies
    // (3 level kernels, 2 moments kernels, captured once here) are added per
    // iteration
    *nlaunch = c->launches - l0 - 5;
    c->launches = l0;
    if (!rc && e != cudaSuccess) rc = cuda_check(c, e, "cudaStreamEndCapture");
    if (!rc) {
        e = cudaGraphInstantiate(exec, g, 0);
        if (e != cudaSuccess) rc = cuda_check(c, e, "cudaGraphInstantiate");
    }
    if (g) cudaGraphDestroy(g);
    return rc;
}

static void drop_step_graphs(Ctx *c)
{
    for (auto &x : c->step_exec)
        if (x) {
            cudaGraphExecDestroy(x);
            x = nullptr;
        }
    c->step_key = 0;
}

// One step as a replay of a captured graph: the same launches as ag2_step, with
// the build's counts kept on the device (the level loop and the moments levels
// are conditional WHILE nodes).  Two graphs, one per state buffer the step
// starts from (the build's reorder swaps them).
static int run_step_graph(Ctx *c, double dt, double hubble, int with_visual, double Rv)
{
    int rc;
    if (c->n == 0) return AG2_OK;
    if ((rc = prepare_captured_build(c)) != AG2_OK) return rc;
    if (c->n_inst == 1 && !c->inst_explicit) {
        AG2_CUDA(c, cudaMemcpy(c->inst_massInH, &c->prm.massInH, sizeof(double), cudaMemcpyHostToDevice));
    }
    if (!c->side_stream) AG2_CUDA(c, cudaStreamCreateWithFlags(&c->side_stream, cudaStreamNonBlocking));
    if (c->inst_R_pin_cap < (size_t)c->n_inst) {
        if (c->inst_R_pin) cudaFreeHost(c->inst_R_pin);
        c->inst_R_pin = nullptr;
        AG2_CUDA(c, cudaMallocHost(&c->inst_R_pin, c->n_inst * sizeof(double)));
        c->inst_R_pin_cap = c->n_inst;
        drop_step_graphs(c);
    }
    const unsigned long long key = step_key(c, dt, hubble, with_visual, Rv);
    if (key != c->step_key || !c->step_exec[c->cur]) {
        drop_step_graphs(c);
        const int cur0 = c->cur;
        for (int p = 0; p < 2 && !rc; p++) {
            c->cur = cur0 ^ p;
            rc = capture_step(c, dt, hubble, with_visual, Rv, &c->step_exec[c->cur], &c->graph_launches[c->cur]);
        }
        c->cur = cur0;
        if (rc) {
            drop_step_graphs(c);
            return rc;
        }
        c->step_key = key;
    }
    const int from = c->cur;
    AG2_CUDA(c, cudaGraphLaunch(c->step_exec[from], c->stream));
    AG2_CUDA(c, cudaStreamSynchronize(c->stream));
    c->cur ^= 1;
    const Ctx::Ctl &h = *c->ctl_host;
    const int mlevels = moments_launches(h.lvl_cnt);
    // the level loop ran once per level it advanced, the moments loop once per launch of its levels
    c->launches += c->graph_launches[from] + 3 * (int64_t)h.level + 2 * (int64_t)mlevels;
    c->inter_grav = (int64_t)h.inter_grav;
    c->inter_sph = (int64_t)h.inter_sph;
    if (h.err_code) {
        c->have_tree = false;
        c->hist_dirty = true;
        switch (h.err_code) {
        case AG2_E_STACK: return set_err(c, AG2_E_STACK, "walk stack overflow (tree deeper than the walk stack supports)");
        case AG2_E_COINCIDENT:
            return set_err(c, AG2_E_COINCIDENT, "particles too close to separate within AG2_MAX_DEPTH levels");
        case AG2_E_NOMEM: return set_err(c, AG2_E_NOMEM, "node pool of the step graph exhausted (redo the step)");
        default: return set_err(c, h.err_code, "captured step failed");
        }
    }
    build_tree_finish_captured(c);
    if (hubble != 1.0) c->have_tree = false;
    return AG2_OK;
}

int ag2_block_init(ag2_ctx *c, double eta, double min_dt, double max_dt, double global_time)
{
    if (!c) return AG2_E_INVALID;
    return run_block_init(c, eta, min_dt, max_dt, global_time);
}

int ag2_block_step(ag2_ctx *c, double H0, int with_visual, double Rv, double *global_time, int64_t *active)
{
    if (!c) return AG2_E_INVALID;
    return run_block_step(c, H0, with_visual, Rv, global_time, active);
}

int ag2_step_graphs(ag2_ctx *c, int enable)
{
    if (!c) return AG2_E_INVALID;
    c->use_graphs = enable != 0;
    if (!c->use_graphs) drop_step_graphs(c);
    return AG2_OK;
}

int ag2_step(ag2_ctx *c, double dt, double hubble_factor, int with_visual, double Rv)
{
    if (!c) return AG2_E_INVALID;
    if (c->use_graphs && !c->timing) return run_step_graph(c, dt, hubble_factor, with_visual, Rv);
    int rc;
    // phase names follow the reference's Log::startProcess calls (Simulation.cpp:256-351)
    phase_reset(c);
    if ((rc = run_kick_drift(c, dt))) return rc;
    phase_mark(c, "first kick");
    const bool t = c->timing;
    c->timing = false;  // the build's own sub-phases are not split inside a step
    rc = build_tree(c);
    c->timing = t;
    if (rc) return rc;
    phase_mark(c, "build tree");
    if (with_visual && (rc = run_visual_density(c, Rv))) return rc;
    phase_mark(c, "Visual Density");
    if ((rc = run_sph_density(c))) return rc;
    phase_mark(c, "SPH density and update");
    AG2_CUDA(c, cudaMemsetAsync(&c->ctl->err_code, 0, sizeof(int32_t), c->stream));
    if ((rc = run_forces(c))) return rc;
    phase_mark(c, "Force Calculation");
    if ((rc = run_close_step(c, dt, hubble_factor))) return rc;
    phase_mark(c, "second kick");
    rc = check_walk(c);
    phase_finish(c);
    return rc;
}

// ag2_upload followed by ag2_set_field(AG2_ACC, acc), the same result bit for
// bit, with the accelerations' host-to-device copy on the copy stream, queued
// behind the other fields' copies: it crosses the link while the slot-order
// gather of those fields runs, instead of after it.
static int upload_with_acc(Ctx *c, size_t n, const double *pos, const double *vel, const double *mass,
                           const double *U, const uint8_t *type, const double *acc)
{
    if (n > c->cap) return set_err(c, AG2_E_CAPACITY, "more particles than the context capacity");
    if (!pos || !mass || !type) return set_err(c, AG2_E_INVALID, "pos, mass and type are required");
    int rc;
    if ((rc = dl_begin(c))) return rc;  // the copy stream
    if (!c->acc_stage) {
        if (cudaMalloc(&c->acc_stage, 3 * c->cap * sizeof(double)) != cudaSuccess) {
            c->acc_stage = nullptr;
            cudaGetLastError();
            return set_err(c, AG2_E_NOMEM, "acceleration staging allocation failed");
        }
        for (auto &e : c->up_ev) AG2_CUDA(c, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    Particles &spare = c->st[1];
    double *pos_d = c->staging, *vel_d = vel ? c->staging + 3 * n : nullptr;
    AG2_CUDA(c, cudaMemcpyAsync(pos_d, pos, 3 * n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    if (vel) AG2_CUDA(c, cudaMemcpyAsync(vel_d, vel, 3 * n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    AG2_CUDA(c, cudaMemcpyAsync(spare.m, mass, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    if (U) AG2_CUDA(c, cudaMemcpyAsync(spare.U, U, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    AG2_CUDA(c, cudaMemcpyAsync(c->staging_u8, type, n, cudaMemcpyHostToDevice, c->stream));
    // the accelerations after those copies (the link is shared), beside the gather
    AG2_CUDA(c, cudaEventRecord(c->up_ev[0], c->stream));
    AG2_CUDA(c, cudaStreamWaitEvent(c->copy_stream, c->up_ev[0], 0));
    AG2_CUDA(c, cudaMemcpyAsync(c->acc_stage, acc, 3 * n * sizeof(double), cudaMemcpyHostToDevice, c->copy_stream));
    AG2_CUDA(c, cudaEventRecord(c->up_ev[1], c->copy_stream));
    rc = upload_common(c, n, pos_d, vel_d, spare.m, U ? spare.U : nullptr, c->staging_u8);
    if (!rc) rc = io_reset_tags(c, n);
    // the scatter waits for the copy; a failure above still has to let it land
    AG2_CUDA(c, cudaStreamWaitEvent(c->stream, c->up_ev[1], 0));
    if (rc) return rc;
    AG2_LAUNCH(c, k_scatter_in, grid_for(n, kBlock), kBlock, 0, (int)n, c->S(), AG2_ACC, c->acc_stage);
    c->graph_epoch++;
    return AG2_OK;
}

// The step itself; ag2_step_host routes every failure through dl_abort, since
// the position and acceleration read-backs start before the step ends.
static int step_host(ag2_ctx *c, size_t n, double dt, double hubble_factor, int with_visual, double Rv,
                     const ag2_host_io *io)
{
    int rc;
    if (io->acc) {
        if ((rc = upload_with_acc(c, n, io->pos, io->vel, io->mass, io->U, io->type, io->acc))) return rc;
    } else if ((rc = ag2_upload(c, n, io->pos, io->vel, io->mass, io->U, io->type))) {
        return rc;
    }
    if (io->first && (rc = ag2_set_instances(c, io->n_inst, io->first, io->massInH))) return rc;
    if ((rc = dl_begin(c))) return rc;
    phase_reset(c);
    if ((rc = run_kick_drift(c, dt))) return rc;
    phase_mark(c, "first kick");
    const bool t = c->timing;
    c->timing = false;
    rc = build_tree(c);
    c->timing = t;
    if (rc) return rc;
    phase_mark(c, "build tree");
    if (with_visual && (rc = run_visual_density(c, Rv))) return rc;
    phase_mark(c, "Visual Density");
    if ((rc = run_sph_density(c))) return rc;
    phase_mark(c, "SPH density and update");
    // positions are final since the drift: their read-back crosses to the host
    // during the walk, which reads nothing back until it ends (the build reads
    // its control block every level, and those small copies would queue behind
    // this one on the device-to-host copy engine)
    int k = 0;
    if (io->pos_out && (rc = dl_field(c, k++, AG2_POS, io->pos_out))) return rc;
    AG2_CUDA(c, cudaMemsetAsync(&c->ctl->err_code, 0, sizeof(int32_t), c->stream));
    if ((rc = run_forces(c))) return rc;
    phase_mark(c, "Force Calculation");
    // accelerations are final after the walk: their copy runs during the
    // closing kick and the internal-energy update
    if (io->acc_out && (rc = dl_field(c, k++, AG2_ACC, io->acc_out))) return rc;
    if ((rc = run_close_step(c, dt, hubble_factor))) return rc;
    phase_mark(c, "second kick");
    if ((rc = check_walk(c))) return rc;
    if (c->inject_site == 1) {  // a failure of the walk's check, as the host sees one (ag2_inject_fault)
        c->inject_site = 0;
        return set_err(c, c->inject_code, "injected failure after the walk");
    }
    if (io->vel_out && (rc = dl_field(c, k++, AG2_VEL, io->vel_out))) return rc;
    if (io->U_out && (rc = dl_field(c, k++, AG2_U, io->U_out))) return rc;
    rc = dl_end(c);
    phase_finish(c);
    return rc;
}

int ag2_step_host(ag2_ctx *c, size_t n, double dt, double hubble_factor, int with_visual, double Rv,
                  const ag2_host_io *io)
{
    if (!c || !io) return AG2_E_INVALID;
    if (n == 0) return set_err(c, AG2_E_INVALID, "no particles");
    const int rc = step_host(c, n, dt, hubble_factor, with_visual, Rv, io);
    return rc ? dl_abort(c, rc) : rc;
}

int ag2_phase_timing(ag2_ctx *c, int enable)
{
    if (!c) return AG2_E_INVALID;
    if (enable && !c->ev[0])
        for (auto &e : c->ev) AG2_CUDA(c, cudaEventCreate(&e));
    c->timing = enable != 0;
    return AG2_OK;
}

int ag2_phase_times(const ag2_ctx *c, int max, const char **names, float *ms)
{
    if (!c || max < 0) return AG2_E_INVALID;
    int k = c->phase_count < max ? c->phase_count : max;
    for (int i = 0; i < k; i++) {
        if (names) names[i] = c->phase_name[i];
        if (ms) ms[i] = c->phase_ms[i];
    }
    return c->phase_count;
}

int ag2_set_instances(ag2_ctx *c, int32_t n_inst, const int64_t *first, const double *massInH)
{
    if (!c || n_inst < 1 || !first) return set_err(c, AG2_E_INVALID, "bad instance layout");
    if (first[0] != 0 || first[n_inst] != (int64_t)c->n)
        return set_err(c, AG2_E_INVALID, "instances must cover the uploaded particles: first[0] = 0, first[k] = n");
    for (int k = 0; k < n_inst; k++)
        if (first[k + 1] < first[k]) return set_err(c, AG2_E_INVALID, "instance offsets must not decrease");
    c->n_inst = n_inst;
    c->inst_first_h.assign(first, first + n_inst + 1);
    c->inst_massInH_h.assign(n_inst, c->prm.massInH);
    if (massInH) c->inst_massInH_h.assign(massInH, massInH + n_inst);
    c->inst_dirty = true;
    c->inst_explicit = true;
    c->have_tree = false;
    c->graph_epoch++;
    return AG2_OK;
}

int ag2_instance_radius(ag2_ctx *c, int32_t k, double *r)
{
    if (!c || !r) return AG2_E_INVALID;
    if (!c->have_tree) return set_err(c, AG2_E_INVALID, "no tree");
    if (k < 0 || k >= c->n_inst) return set_err(c, AG2_E_INVALID, "no such instance");
    *r = c->inst_R_h[k];
    return AG2_OK;
}

int ag2_root_radius(ag2_ctx *c, double *r)
{
    if (!c || !r) return AG2_E_INVALID;
    if (!c->have_tree) return set_err(c, AG2_E_INVALID, "no tree");
    *r = c->root_radius;
    return AG2_OK;
}

int ag2_node_count(ag2_ctx *c, int64_t *nodes, int64_t *internal, int32_t *max_depth)
{
    if (!c) return AG2_E_INVALID;
    if (!c->have_tree) return set_err(c, AG2_E_INVALID, "no tree");
    if (nodes) *nodes = c->nnodes_true;
    if (internal) *internal = c->ninternal;
    if (max_depth) *max_depth = c->max_level;
    return AG2_OK;
}

int ag2_interactions(ag2_ctx *c, int64_t *g, int64_t *s)
{
    if (!c) return AG2_E_INVALID;
    if (g) *g = c->inter_grav;
    if (s) *s = c->inter_sph;
    return AG2_OK;
}

int64_t ag2_launch_count(const ag2_ctx *c) { return c ? c->launches : 0; }

int ag2_direct_sum(ag2_ctx *c, size_t ns, const int64_t *ids, double *out)
{
    if (!c || (ns && (!ids || !out))) return AG2_E_INVALID;
    return run_direct_sum(c, ns, ids, out);
}

int ag2_autotune(ag2_ctx *c, int *variant)
{
    if (!c || !variant) return AG2_E_INVALID;
    AG2_CUDA(c, cudaMemsetAsync(&c->ctl->err_code, 0, sizeof(int32_t), c->stream));
    int rc = run_autotune(c, variant);
    if (rc) return rc;
    return check_walk(c);
}

int ag2_set_walk_variant(ag2_ctx *c, int variant)
{
    if (!c || variant < 0 || variant >= kWalkVariantCount) return AG2_E_INVALID;
    c->walk_variant = variant;
    c->graph_epoch++;
    return AG2_OK;
}

int ag2_autotune_walk(ag2_ctx *c, int max, ag2_walk_config *out, int *count, int *chosen)
{
    if (!c || !chosen || max < 0 || (max > 0 && !out)) return AG2_E_INVALID;
    AG2_CUDA(c, cudaMemsetAsync(&c->ctl->err_code, 0, sizeof(int32_t), c->stream));
    int variant = 0, k = 0;
    int rc = run_autotune(c, &variant, out, max, &k);
    if (rc) return rc;
    if (count) *count = k;
    *chosen = -1;
    for (int j = 0; j < std::min(k, max); j++)
        if (out[j].variant == variant && out[j].group_size == c->prm.group_size) *chosen = j;
    return check_walk(c);
}

int ag2_diagnostics(ag2_ctx *c, double *out8)
{
    if (!c || !out8) return AG2_E_INVALID;
    return run_diagnostics(c, out8);
}

int ag2_energy(ag2_ctx *c, double *out4)
{
    if (!c || !out4) return AG2_E_INVALID;
    return run_energy(c, out4);
}

int ag2_fp32_peak_probe(ag2_ctx *c, double *gflops)
{
    if (!c || !gflops) return AG2_E_INVALID;
    return run_fma_probe(c, gflops);
}

static uint64_t id_hash(uint64_t id)
{
    uint64_t z = id + 1 + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

int ag2_particle_node(ag2_ctx *c, int64_t *out)
{
    if (!c || !out) return AG2_E_INVALID;
    if (!c->have_tree) return set_err(c, AG2_E_INVALID, "no tree");
    const int64_t nn = c->nnodes;
    const size_t n = c->n;
    std::vector<int32_t> first(nn), ref(n), id(n);
    AG2_CUDA(c, cudaMemcpyAsync(first.data(), c->nd.first, nn * 4, cudaMemcpyDeviceToHost, c->stream));
    if (n) {
        AG2_CUDA(c, cudaMemcpyAsync(ref.data(), c->refnode, n * 4, cudaMemcpyDeviceToHost, c->stream));
        AG2_CUDA(c, cudaMemcpyAsync(id.data(), c->S().id, n * 4, cudaMemcpyDeviceToHost, c->stream));
    }
    AG2_CUDA(c, cudaStreamSynchronize(c->stream));
    std::vector<int64_t> pre(nn, -1), stack;
    for (int r = c->n_inst - 1; r >= 0; r--) stack.push_back(r);
    int64_t k = 0;
    while (!stack.empty()) {
        int64_t v = stack.back();
        stack.pop_back();
        pre[v] = k++;
        if (first[v] >= 0)
            for (int o = 7; o >= 0; o--) stack.push_back(first[v] + o);
    }
    for (size_t i = 0; i < n; i++) out[id[i]] = ref[i] >= 0 ? pre[ref[i]] : -1;
    return AG2_OK;
}

int ag2_walk_records(ag2_ctx *c, float *out16)
{
    if (!c || !out16) return AG2_E_INVALID;
    if (!c->have_tree) return set_err(c, AG2_E_INVALID, "no tree");
    const int64_t nn = c->nnodes;
    std::vector<int32_t> first(nn), count(nn);
    std::vector<WalkRec> rec(nn);
    AG2_CUDA(c, cudaMemcpyAsync(first.data(), c->nd.first, nn * 4, cudaMemcpyDeviceToHost, c->stream));
    AG2_CUDA(c, cudaMemcpyAsync(count.data(), c->nd.count, nn * 4, cudaMemcpyDeviceToHost, c->stream));
    AG2_CUDA(c, cudaMemcpyAsync(rec.data(), c->nd.wrec, nn * sizeof(WalkRec), cudaMemcpyDeviceToHost, c->stream));
    AG2_CUDA(c, cudaStreamSynchronize(c->stream));
    std::vector<int64_t> stack;
    for (int r = c->n_inst - 1; r >= 0; r--) stack.push_back(r);
    int64_t k = 0;
    while (!stack.empty()) {
        const int64_t v = stack.back();
        stack.pop_back();
        float *o = out16 + 16 * k++;
        if (count[v] > 0)
            std::memcpy(o, &rec[v], sizeof(WalkRec));
        else
            std::memset(o, 0, sizeof(WalkRec));
        if (first[v] >= 0)
            for (int q = 7; q >= 0; q--) stack.push_back(first[v] + q);
    }
    return AG2_OK;
}

int ag2_topology(ag2_ctx *c, int32_t *depth, int32_t *is_leaf, int32_t *particle, int64_t *cp_count,
                 uint64_t *cp_hash, double *mass, double *com3, double *gas_mass, double *mvel3, double *center3,
                 double *radius)
{
    if (!c) return AG2_E_INVALID;
    if (!c->have_tree) return set_err(c, AG2_E_INVALID, "no tree");
    const int64_t nn = c->nnodes;
    const size_t n = c->n;
    std::vector<int32_t> start(nn), count(nn), ndrop(nn), first(nn), leafpos(nn), id(n);
    std::vector<int8_t> level(nn);
    std::vector<uint8_t> mode(nn);
    std::vector<double> m(nn), cx(nn), cy(nn), cz(nn), g(nn), vx(nn), vy(nn), vz(nn), ccx(nn), ccy(nn), ccz(nn);
    std::vector<int32_t> inst_of(nn), parent(nn);
    std::vector<double> rad(nn);
    auto cp = [&](void *dst, const void *src, size_t bytes) {
        return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, c->stream);
    };
    Nodes &d = c->nd;
    AG2_CUDA(c, cp(start.data(), d.start, nn * 4));
    AG2_CUDA(c, cp(count.data(), d.count, nn * 4));
    AG2_CUDA(c, cp(ndrop.data(), d.ndrop, nn * 4));
    AG2_CUDA(c, cp(first.data(), d.first, nn * 4));
    AG2_CUDA(c, cp(leafpos.data(), d.leafpos, nn * 4));
    AG2_CUDA(c, cp(level.data(), d.level, nn));
    AG2_CUDA(c, cp(mode.data(), d.mode, nn));
    // one field of every NodeMom record: a strided copy
    auto cpm = [&](double *dst, size_t field) {
        return cudaMemcpy2DAsync(dst, sizeof(double), reinterpret_cast<const char *>(d.mom) + field * sizeof(double),
                                 sizeof(NodeMom), sizeof(double), nn, cudaMemcpyDeviceToHost, c->stream);
    };
    AG2_CUDA(c, cpm(m.data(), 0));
    AG2_CUDA(c, cpm(cx.data(), 1));
    AG2_CUDA(c, cpm(cy.data(), 2));
    AG2_CUDA(c, cpm(cz.data(), 3));
    AG2_CUDA(c, cpm(g.data(), 4));
    AG2_CUDA(c, cpm(vx.data(), 5));
    AG2_CUDA(c, cpm(vy.data(), 6));
    AG2_CUDA(c, cpm(vz.data(), 7));
    AG2_CUDA(c, cp(ccx.data(), d.cx, nn * 8));
    AG2_CUDA(c, cp(ccy.data(), d.cy, nn * 8));
    AG2_CUDA(c, cp(ccz.data(), d.cz, nn * 8));
    AG2_CUDA(c, cp(inst_of.data(), d.inst, nn * 4));
    AG2_CUDA(c, cp(parent.data(), d.parent, nn * 4));
    AG2_CUDA(c, cp(rad.data(), d.radius, nn * 8));
    if (n) AG2_CUDA(c, cp(id.data(), c->S().id, n * 4));
    AG2_CUDA(c, cudaStreamSynchronize(c->stream));
    // prefix sums of member hashes over tree-order slots
    std::vector<uint64_t> hp(n + 1, 0);
    for (size_t i = 0; i < n; i++) hp[i + 1] = hp[i] + id_hash((uint64_t)id[i]);
    auto hsum = [&](int32_t a, int32_t b) { return hp[b] - hp[a]; };
    // depth-first preorder, children 0..7, instance after instance
    std::vector<int64_t> stack;
    for (int r = c->n_inst - 1; r >= 0; r--) stack.push_back(r);
    int64_t k = 0;
    while (!stack.empty()) {
        int64_t v = stack.back();
        stack.pop_back();
        int32_t s = start[v], e = s + count[v], re = e - ndrop[v];
        int64_t cc = 0;
        uint64_t ch = 0;
        bool root = (v < c->n_inst);
        switch (mode[v]) {
        case MODE_PAR:
        case MODE_VEC1:
            if (!root) { cc = e - s; ch = hsum(s, e); }
            break;
        case MODE_SER_ENTRY:
            if (root) { cc = re - s; ch = hsum(s, re); }
            else { cc = (e - s) + (re - s); ch = hsum(s, e) + hsum(s, re); }
            break;
        case MODE_SER:
            cc = re - s;
            ch = hsum(s, re);
            break;
        default:
            break;
        }
        if (depth) depth[k] = level[v];
        if (is_leaf) is_leaf[k] = first[v] < 0 ? 1 : 0;
        if (particle) particle[k] = leafpos[v] >= 0 ? id[leafpos[v]] : -1;
        if (cp_count) cp_count[k] = cc;
        if (cp_hash) cp_hash[k] = ch;
        const bool empty = count[v] == 0;  // the build leaves empty children's moments unwritten
        if (empty && !root) {
            // nor their centres: parent centre + r*(+-0.5), as for every child (Node.cpp:433-443)
            const int32_t pa = parent[v];
            const int o = (int)(v - first[pa]);
            const double rc = rad[pa] / 2;
            ccx[v] = ccx[pa] + ((o & 1) ? rc : -rc);
            ccy[v] = ccy[pa] + ((o & 2) ? rc : -rc);
            ccz[v] = ccz[pa] + ((o & 4) ? rc : -rc);
        }
        if (mass) mass[k] = empty ? 0.0 : m[v];
        if (com3) {
            com3[3 * k] = empty ? 0.0 : cx[v];
            com3[3 * k + 1] = empty ? 0.0 : cy[v];
            com3[3 * k + 2] = empty ? 0.0 : cz[v];
        }
        if (gas_mass) gas_mass[k] = empty ? 0.0 : g[v];
        if (mvel3) {
            mvel3[3 * k] = empty ? 0.0 : vx[v];
            mvel3[3 * k + 1] = empty ? 0.0 : vy[v];
            mvel3[3 * k + 2] = empty ? 0.0 : vz[v];
        }
        if (center3) { center3[3 * k] = ccx[v]; center3[3 * k + 1] = ccy[v]; center3[3 * k + 2] = ccz[v]; }
        if (radius) radius[k] = std::ldexp(c->inst_R_h[c->n_inst == 1 ? 0 : inst_of[v]], -(int)level[v]);
        k++;
        if (first[v] >= 0)
            for (int o = 7; o >= 0; o--) stack.push_back(first[v] + o);
    }
    return AG2_OK;
}

}  // extern "C"
