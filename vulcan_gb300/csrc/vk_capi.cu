// C ABI: handle life cycle, uploads and the Ros2 attempt pipeline.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include <chrono>
#include <climits>
#include <cmath>

#include "vk_control.cuh"
#include "vk_internal.cuh"

namespace vk {
void launch_chem_only(const DevNet &net, const DevBatch &b, const double *y, double *f,
                      const double *geo, cudaStream_t s);
cudaError_t init_kernels(const DevNet &net);
}

struct vk_handle {
    std::string err;
    int ni = 0, npair = 0, nr = 0, nnz = 0, nw = 0, natom = 0;
    int max_cols = 0, max_layers = 0, precision = VK_PREC_FP64;
    int max_refine = 6;
    double refine_tol = 1e-10;
    double route_dt0 = INFINITY;  // vk_set_route: FP64 from this step size until a failure lowers it
    int geo_flags = -1;         // flags the transport geometry was built for (-1: stale)
    CUtensorMap tmap_d32{};     // k_lu_tc's view of w.D32 (mixed mode, ni <= 128)
    int ncols = 0, L = 0;
    std::vector<int> col_off, col_end;  // first / one past last layer of each column
    int slot_cap = 0;                   // > 0: slotted layout (vk_set_columns_slotted)
    // network tables
    PairDesc *d_pairs = nullptr;
    int *d_src_ptr = nullptr;
    int *d_src_order = nullptr;
    int *d_jorder = nullptr;
    int2 *d_src = nullptr;
    double *d_src_nu = nullptr, *d_jterm_nu = nullptr;
    WDesc *d_w = nullptr;
    int *d_jptr = nullptr;
    int2 *d_jterm = nullptr;
    int *d_jpos = nullptr;
    int *d_jrow = nullptr, *d_jcol = nullptr, *d_jrowptr = nullptr, *d_jmap = nullptr;
    double *d_compo = nullptr;
    int nxm = 0, nh = 0;                // extra source products, derivative half terms
    int *d_porder = nullptr, *d_src_slot = nullptr, *d_xmul_pair = nullptr;
    double *d_src_c = nullptr, *d_xmul_fac = nullptr, *d_hjcoef = nullptr;
    int *d_hk = nullptr, *d_hptr = nullptr, *d_hjterm = nullptr, *d_hjptr = nullptr;
    int16_t *d_hfac = nullptr;
    // batch
    int *d_col_off = nullptr, *d_col_end = nullptr, *d_lay_col = nullptr;
    int *d_cols = nullptr;              // [max_cols] column list of reset_columns
    int *d_order = nullptr;             // columns by decreasing nz
    PhotoDev ph{};                  // radiative transfer (vk_photo_setup)
    int *d_phmask = nullptr;            // [max_cols] columns of a masked photo update
    std::vector<double> ph_jw;          // J bin weights (host copy, weights cross_J_T)
    int *d_abs_tslot = nullptr, *d_ch_tslot = nullptr;   // vk_photo_set_cross_T
    double *d_crossT = nullptr, *d_wcrossJT = nullptr;
    int tcap_abs = 0, tcap_ch = 0;      // table rows allocated
    int *d_kkind = nullptr, *d_krev = nullptr;   // rate-constant parameters (vk_set_rate_params)
    double *d_kpar = nullptr, *d_nasa9 = nullptr;
    int *d_capk = nullptr;              // low-temperature caps (vk_set_rate_caps)
    double *d_capT = nullptr, *d_capp = nullptr;
    int caps_on = 0;
    unsigned *d_queue = nullptr;        // work-queue position of the per-column kernels
    unsigned *d_queue2 = nullptr;       // the same for the FP64 branch of a mixed attempt
    cudaStream_t stream2 = nullptr;     // FP64 branch of a mixed attempt (routed columns)
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    int nsm = 0;                        // SMs of the device
    int cps = 0;                        // VK_CTAS_PER_SM override (0: kernel defaults)
    int cps_k[VK_TUNE_N] = {0, 0, 0, 0}; // vk_set_launch: CTAs per SM per kernel
    int lu32_tiling = -1;               // vk_set_launch: k_lu32 tiling (-1: by ni)
    int occ_rates = 0, occ_prep = 0;    // resident CTAs per SM of k_rates / k_prep32
    double *d_k = nullptr, *d_atm = nullptr, *d_Dzz = nullptr, *d_spf = nullptr;
    vk::Work w{};
    // batched-run state
    vk::RunState rs{};
    int rs_ready = 0;           // run-state buffers allocated
    int hist_R = 0;             // ring length the history was sized for
    int *d_nactive = nullptr;
    cudaGraphExec_t gexec = nullptr;
    unsigned char gkey[sizeof(vk::RunCtrl) + 2 * sizeof(int)] = {};
    unsigned gen = 0;           // bumped whenever a captured loop of this handle goes stale
    std::vector<void *> allocs;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[8] = {};
    float ms[4] = {0, 0, 0, 0};
    int launches = 0;

    DevNet net() const {
        DevNet n;
        n.ni = ni; n.npair = npair; n.nr = nr; n.nw = nw; n.nnz = nnz; n.natom = natom;
        n.pairs = d_pairs; n.src_ptr = d_src_ptr; n.src = d_src; n.w = d_w;
        n.src_order = d_src_order; n.jorder = d_jorder;
        n.src_nu = d_src_nu; n.jterm_nu = d_jterm_nu;
        n.jptr = d_jptr; n.jterm = d_jterm; n.jpos = d_jpos; n.compo = d_compo;
        n.jrow = d_jrow; n.jcol = d_jcol; n.jrowptr = d_jrowptr; n.jmap = d_jmap;
        n.nxm = nxm; n.nh = nh; n.porder = d_porder; n.src_slot = d_src_slot; n.src_c = d_src_c;
        n.xmul_pair = d_xmul_pair; n.xmul_fac = d_xmul_fac; n.hk = d_hk; n.hptr = d_hptr;
        n.hfac = d_hfac; n.hjterm = d_hjterm; n.hjptr = d_hjptr; n.hjcoef = d_hjcoef;
        return n;
    }
    DevBatch batch() const {
        DevBatch b;
        b.ncols = ncols; b.L = L; b.col_off = d_col_off; b.col_end = d_col_end; b.lay_col = d_lay_col;
        b.k = d_k; b.atm = d_atm; b.Dzz = d_Dzz; b.spf = d_spf;
        b.active = nullptr;
        b.order = d_order;
        b.queue = d_queue;
        b.nsm = nsm;
        b.cps = cps;
        for (int i = 0; i < VK_TUNE_N; ++i) b.cps_k[i] = cps_k[i];
        b.lu32_tiling = lu32_tiling;
        b.grid_rates = nsm * occ_rates;
        b.grid_prep = nsm * occ_prep;
        return b;
    }
};

static thread_local std::string g_err;

void vk::set_global_error(const std::string &msg) { g_err = msg; }

static int fail(vk_handle *h, int code, const std::string &msg) {
    if (h) h->err = msg; else g_err = msg;
    return code;
}

#define VK_CUDA(h, call)                                                              \
    do {                                                                              \
        cudaError_t e_ = (call);                                                      \
        if (e_ != cudaSuccess)                                                        \
            return fail((h), VK_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

template <typename T>
static int dalloc(vk_handle *h, T **p, size_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc((void **)p, count * sizeof(T));
    if (e != cudaSuccess) {
        *p = nullptr;
        return fail(h, VK_ENOMEM, std::string("cudaMalloc of ") + std::to_string(count * sizeof(T)) +
                                      " bytes: " + cudaGetErrorString(e));
    }
    h->allocs.push_back((void *)*p);
    return VK_OK;
}

static void dfree(vk_handle *h, void *p) {
    if (!p) return;
    for (size_t i = 0; i < h->allocs.size(); ++i)
        if (h->allocs[i] == p) {
            h->allocs.erase(h->allocs.begin() + (long)i);
            break;
        }
    cudaFree(p);
}

template <typename T>
static int upload(vk_handle *h, T **p, const std::vector<T> &v) {
    int rc = dalloc(h, p, v.size());
    if (rc) return rc;
    if (!v.empty()) VK_CUDA(h, cudaMemcpy(*p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    return VK_OK;
}

// A captured run loop of h (its own, or a group's that holds h) no longer
// matches the handle's buffers, grids or precision settings.
static void drop_graph(vk_handle *h) {
    if (h->gexec) { cudaGraphExecDestroy(h->gexec); h->gexec = nullptr; }
    ++h->gen;
}

extern "C" const char *vk_last_error(const vk_handle *h) {
    return h ? h->err.c_str() : g_err.c_str();
}

extern "C" void vk_destroy(vk_handle *h) {
    if (!h) return;
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (h->gexec) cudaGraphExecDestroy(h->gexec);
    if (h->rs.hist_y) cudaFree(h->rs.hist_y);
    if (h->rs.hist_t) cudaFree(h->rs.hist_t);
    for (void *p : h->allocs) cudaFree(p);
    for (auto &e : h->ev) if (e) cudaEventDestroy(e);
    if (h->ev_fork) cudaEventDestroy(h->ev_fork);
    if (h->ev_join) cudaEventDestroy(h->ev_join);
    if (h->stream2) cudaStreamDestroy(h->stream2);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
}

// Buffers of the mixed-precision path: the FP32 inverses (packed n x n per
// layer) and the scaled blocks, sized for k_lu32's packed layout or k_lu_tc's
// zero-padded NP x NP tiles, with the tensor map k_lu_tc loads them through.
static int alloc_mixed(vk_handle *h) {
    const size_t st = (size_t)((h->ni * h->ni + 3) & ~3);
    const bool tc = vk::lu_tc_supported(h->ni);
    const size_t sd = tc ? std::max(st, vk::lu_tc_block_floats(h->ni)) : st;
    const size_t lv = (size_t)h->max_layers * h->ni;
    int rc = dalloc(h, &h->w.G32, (size_t)h->max_layers * st);
    if (!rc) rc = dalloc(h, &h->w.D32, (size_t)h->max_layers * sd);
    if (!rc) rc = dalloc(h, &h->w.wcf, lv);
    if (!rc) rc = dalloc(h, &h->w.wcb, lv);
    if (!rc) rc = dalloc(h, &h->w.raf, lv);
    if (!rc) rc = dalloc(h, &h->w.xf, lv);
    if (rc) return rc;
    if (tc) {
        cudaError_t e = vk::lu_tc_make_map(&h->tmap_d32, h->w.D32, h->ni, h->max_layers);
        if (e != cudaSuccess)
            return fail(h, VK_ECUDA, std::string("tensor map of the scaled blocks: ") + cudaGetErrorString(e));
        h->w.tmap_d32 = &h->tmap_d32;
    }
    return VK_OK;
}

extern "C" int vk_create(const vk_network *net, int max_cols, int max_layers, int precision,
                         vk_handle **out) {
    if (!out) return fail(nullptr, VK_EINVAL, "out is NULL");
    *out = nullptr;
    if (!net) return fail(nullptr, VK_EINVAL, "network is NULL");
    if (max_cols <= 0 || max_layers < 2 * max_cols)
        return fail(nullptr, VK_EINVAL, "need max_cols > 0 and max_layers >= 2*max_cols");
    if (precision != VK_PREC_FP64 && precision != VK_PREC_MIXED)
        return fail(nullptr, VK_EINVAL, "unknown precision mode");
    vk_handle *h = new (std::nothrow) vk_handle();
    if (!h) return fail(nullptr, VK_ENOMEM, "host allocation failed");
    h->ni = net->ni; h->npair = net->npair; h->nr = 2 * net->npair;
    h->nnz = (int)net->jpos.size(); h->nw = (int)net->w.size(); h->natom = net->natom;
    h->max_cols = max_cols; h->max_layers = max_layers; h->precision = precision;
    int rc = VK_OK;
#define TRY(x) do { rc = (x); if (rc) { g_err = h->err; vk_destroy(h); return rc; } } while (0)
    {
        cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) {
            g_err = std::string("cudaStreamCreate: ") + cudaGetErrorString(e);
            delete h;
            return VK_ECUDA;
        }
    }
    for (auto &e : h->ev) TRY(cudaEventCreate(&e) == cudaSuccess ? VK_OK : fail(h, VK_ECUDA, "cudaEventCreate"));
    TRY(upload(h, &h->d_pairs, net->pairs));
    TRY(upload(h, &h->d_src_ptr, net->src_ptr));
    {
        // the source gather runs one thread per species in the reference's
        // summation order; sorting species by term count gives every warp
        // chains of similar length (FP64 issue is per warp, idle lanes cost)
        std::vector<int> order(h->ni);
        for (int i = 0; i < h->ni; ++i) order[i] = i;
        std::stable_sort(order.begin(), order.end(), [&](int a, int b2) {
            return net->src_ptr[a + 1] - net->src_ptr[a] > net->src_ptr[b2 + 1] - net->src_ptr[b2];
        });
        TRY(upload(h, &h->d_src_order, order));
    }
    TRY(upload(h, &h->d_src, net->src));
    TRY(upload(h, &h->d_src_nu, net->src_nu));
    TRY(upload(h, &h->d_jterm_nu, net->jterm_nu));
    TRY(upload(h, &h->d_w, net->w));
    TRY(upload(h, &h->d_jptr, net->jptr));
    {
        // Jacobian entries by decreasing term count (the same reason)
        const int nnz = (int)net->jptr.size() - 1;
        std::vector<int> order(nnz > 0 ? nnz : 1, 0);
        for (int i = 0; i < nnz; ++i) order[i] = i;
        std::stable_sort(order.begin(), order.begin() + (nnz > 0 ? nnz : 0), [&](int a, int b2) {
            return net->hjptr[a + 1] - net->hjptr[a] > net->hjptr[b2 + 1] - net->hjptr[b2];
        });
        TRY(upload(h, &h->d_jorder, order));
    }
    TRY(upload(h, &h->d_jterm, net->jterm));
    TRY(upload(h, &h->d_jpos, net->jpos));
    TRY(upload(h, &h->d_compo, net->compo));
    TRY(upload(h, &h->d_jrow, net->jrow));
    TRY(upload(h, &h->d_jcol, net->jcol));
    TRY(upload(h, &h->d_jrowptr, net->jrowptr));
    TRY(upload(h, &h->d_jmap, net->jmap));
    h->nxm = (int)net->xmul_pair.size();
    h->nh = (int)net->hk.size();
    TRY(upload(h, &h->d_porder, net->porder));
    TRY(upload(h, &h->d_src_slot, net->src_slot));
    TRY(upload(h, &h->d_src_c, net->src_c));
    TRY(upload(h, &h->d_xmul_pair, net->xmul_pair));
    TRY(upload(h, &h->d_xmul_fac, net->xmul_fac));
    TRY(upload(h, &h->d_hk, net->hk));
    TRY(upload(h, &h->d_hptr, net->hptr));
    TRY(upload(h, &h->d_hfac, net->hfac));
    TRY(upload(h, &h->d_hjterm, net->hjterm));
    TRY(upload(h, &h->d_hjcoef, net->hjcoef));
    TRY(upload(h, &h->d_hjptr, net->hjptr));
    const size_t L = (size_t)max_layers, ni = (size_t)h->ni;
    TRY(dalloc(h, &h->d_col_off, max_cols + 1));
    TRY(dalloc(h, &h->d_col_end, max_cols));
    TRY(dalloc(h, &h->d_cols, max_cols));
    TRY(dalloc(h, &h->d_order, max_cols));
    TRY(dalloc(h, &h->d_queue, 1));
    TRY(dalloc(h, &h->d_queue2, 1));
    TRY(cudaStreamCreateWithFlags(&h->stream2, cudaStreamNonBlocking) == cudaSuccess
            ? VK_OK : fail(h, VK_ECUDA, "cudaStreamCreate (FP64 branch)"));
    TRY(cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming) == cudaSuccess
            ? VK_OK : fail(h, VK_ECUDA, "cudaEventCreate"));
    TRY(cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming) == cudaSuccess
            ? VK_OK : fail(h, VK_ECUDA, "cudaEventCreate"));
    {
        // per-column kernels: k resident CTAs per SM take columns from the queue;
        // k = VK_CTAS_PER_SM when set, else each kernel's measured best
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&h->nsm, cudaDevAttrMultiProcessorCount, dev);
        const char *env = getenv("VK_CTAS_PER_SM");
        h->cps = env ? atoi(env) : 0;
    }
    TRY(dalloc(h, &h->d_lay_col, L));
    TRY(dalloc(h, &h->d_k, L * h->nr));
    TRY(dalloc(h, &h->d_atm, L * VK_ATM_NF));
    TRY(dalloc(h, &h->d_Dzz, L * ni));
    TRY(dalloc(h, &h->d_spf, (size_t)max_cols * VK_SP_NF * ni));
    vk::Work &w = h->w;
    double **vecs[] = {&w.y, &w.ymix, &w.yk2, &w.f, &w.k1, &w.k2, &w.z, &w.sol, &w.ymix_out,
                       &w.dA, &w.dB, &w.dC, &w.r, &w.f2, &w.rs, &w.cs};
    for (double **p : vecs) TRY(dalloc(h, p, L * ni));
    TRY(dalloc(h, &w.jv, L * (size_t)std::max(h->nnz, 1)));
    TRY(dalloc(h, &w.geo, L * 5 * ni));
    // FP64 inverses always (the mixed path falls back to them per column)
    TRY(dalloc(h, &w.G, L * (size_t)block_stride64(ni)));
    if (precision == VK_PREC_MIXED) TRY(alloc_mixed(h));
    TRY(dalloc(h, &w.zf, L * ni));
    TRY(dalloc(h, &w.fallback, max_cols));
    TRY(dalloc(h, &w.act32, max_cols));
    TRY(dalloc(h, &w.routed, max_cols));
    TRY(dalloc(h, &w.failed, max_cols));
    TRY(dalloc(h, &w.thr64, max_cols));
    TRY(dalloc(h, &w.sweeps, 1));
    TRY(dalloc(h, &w.refine_err, max_cols));
    TRY(dalloc(h, &w.dt, max_cols));
    TRY(dalloc(h, &w.delta, max_cols));
    TRY(dalloc(h, &w.status, max_cols));
    TRY(vk::init_kernels(h->net()) == cudaSuccess ? VK_OK
                                                  : fail(h, VK_ECUDA, "cudaFuncSetAttribute failed"));
    TRY(vk::init_mixed_kernels(h->ni) == cudaSuccess ? VK_OK
                                                     : fail(h, VK_ECUDA, "cudaFuncSetAttribute (mixed) failed"));
    TRY(vk::init_lureg_kernels(h->net()) == cudaSuccess ? VK_OK
                                                     : fail(h, VK_ECUDA, "cudaFuncSetAttribute (LU) failed"));
    TRY(vk::init_lu_tc(h->ni) == cudaSuccess ? VK_OK
                                             : fail(h, VK_ECUDA, "cudaFuncSetAttribute (tensor-core LU) failed"));
    h->occ_rates = vk::rates_blocks_per_sm(h->net());
    h->occ_prep = vk::prep_blocks_per_sm(h->net());
    cudaGetLastError();                 // an occupancy query that failed leaves one CTA per layer
    // per-column run state (small); the history ring is sized at the first vk_run
    vk::RunState &r = h->rs;
    r.y = w.y; r.ymix = w.ymix; r.dt = w.dt; r.delta = w.delta; r.atm = h->d_atm;
    TRY(dalloc(h, &r.y_prev, L * ni));
    double **cd[] = {&r.t, &r.longdy, &r.longdydt, &r.aflux_change};
    for (double **p : cd) TRY(dalloc(h, p, max_cols));
    int **ci[] = {&r.count, &r.end_case, &r.active, &r.natt, &r.steps_call, &r.pref};
    for (int **p : ci) TRY(dalloc(h, p, max_cols));
    TRY(dalloc(h, &r.counters, (size_t)max_cols * VK_NCOUNTERS));
    TRY(dalloc(h, &r.atom_ini, (size_t)max_cols * VK_MAX_NATOM));
    TRY(dalloc(h, &r.loss, (size_t)max_cols * VK_MAX_NATOM));
    TRY(dalloc(h, &r.loss_prev, (size_t)max_cols * VK_MAX_NATOM));
    TRY(dalloc(h, &r.ignore, (size_t)max_cols * ni));
    TRY(dalloc(h, &h->d_nactive, 1));
    TRY(cudaMemset(r.ignore, 0, (size_t)max_cols * ni * sizeof(int)) == cudaSuccess ? VK_OK
                                                                               : fail(h, VK_ECUDA, "memset"));
#undef TRY
    *out = h;
    return VK_OK;
}

extern "C" int vk_set_precision(vk_handle *h, int precision, int max_refine, double refine_tol) {
    if (!h) return fail(nullptr, VK_EINVAL, "handle is NULL");
    if (precision == VK_PREC_MIXED && !h->w.G32) {
        int rc = alloc_mixed(h);
        if (rc) return rc;
    }
    if (precision != VK_PREC_FP64 && precision != VK_PREC_MIXED)
        return fail(h, VK_EINVAL, "unknown precision mode");
    if (max_refine < 0 || max_refine > 20) return fail(h, VK_EINVAL, "max_refine out of range");
    h->precision = precision;
    h->max_refine = max_refine;
    h->refine_tol = refine_tol;
    drop_graph(h);
    return VK_OK;
}

extern "C" int vk_set_route(vk_handle *h, double dt0) {
    if (!h) return fail(nullptr, VK_EINVAL, "handle is NULL");
    if (!(dt0 > 0.0)) return fail(h, VK_EINVAL, "dt0 must be positive (INFINITY: no initial limit)");
    h->route_dt0 = dt0;
    if (h->w.thr64 && h->max_cols > 0) {
        vk::launch_reset_route(h->w, h->max_cols, dt0, h->stream);
        VK_CUDA(h, cudaGetLastError());
        VK_CUDA(h, cudaStreamSynchronize(h->stream));
    }
    return VK_OK;
}

// Per-column start of a run (clock, counters, conservation reference,
// routing threshold, dt = 1e-10) of the columns cs, by one kernel.
static int reset_columns(vk_handle *h, const std::vector<int> &cs) {
    if (cs.empty()) return VK_OK;
    cudaStream_t s = h->stream;
    VK_CUDA(h, cudaMemcpyAsync(h->d_cols, cs.data(), cs.size() * sizeof(int), cudaMemcpyHostToDevice, s));
    vk::launch_reset_columns(h->rs, (int)cs.size(), h->d_cols, h->w.dt, h->w.status, h->w.thr64,
                             h->route_dt0, s);
    VK_CUDA(h, cudaGetLastError());
    VK_CUDA(h, cudaStreamSynchronize(s));      // cs may be a temporary
    return VK_OK;
}

// Longest columns first: the work queue then balances the SMs.
static int upload_order(vk_handle *h) {
    std::vector<int> order(h->ncols);
    for (int c = 0; c < h->ncols; ++c) order[c] = c;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b2) {
        return h->col_end[a] - h->col_off[a] > h->col_end[b2] - h->col_off[b2];
    });
    VK_CUDA(h, cudaMemcpy(h->d_order, order.data(), h->ncols * sizeof(int), cudaMemcpyHostToDevice));
    return VK_OK;
}

// Packed (slot_cap 0: column c at the layers after column c-1) or slotted
// (column c at layers c * slot_cap .. + nz[c], the rest of the slot gap
// layers) set-up of every column from packed host arrays.
static int set_columns_impl(vk_handle *h, int ncols, int slot_cap, const int *nz, const double *k,
                            const double *atm, const double *Dzz, const double *spf,
                            const double *y, const double *ymix) {
    if (!h) return fail(nullptr, VK_EINVAL, "handle is NULL");
    if (ncols <= 0 || ncols > h->max_cols)
        return fail(h, VK_EINVAL, "ncols must be in 1.." + std::to_string(h->max_cols));
    if (!nz || !k || !atm || !Dzz || !spf || !y || !ymix)
        return fail(h, VK_EINVAL, "NULL input array");
    if (slot_cap < 0 || slot_cap > 1024) return fail(h, VK_EINVAL, "slot_cap must be in 0..1024");
    std::vector<int> off(ncols + 1, 0), end(ncols, 0), pk(ncols + 1, 0);
    for (int c = 0; c < ncols; ++c) {
        if (nz[c] < 2 || nz[c] > 1024) return fail(h, VK_EINVAL, "every column needs 2 <= nz <= 1024");
        if (slot_cap && nz[c] > slot_cap)
            return fail(h, VK_EINVAL, "column " + std::to_string(c) + " has more layers than slot_cap");
        pk[c + 1] = pk[c] + nz[c];
        off[c + 1] = slot_cap ? (c + 1) * slot_cap : pk[c + 1];
        end[c] = off[c] + nz[c];
        if (off[c + 1] > h->max_layers)
            return fail(h, VK_EINVAL, "total layers exceed max_layers=" + std::to_string(h->max_layers));
    }
    const int L = off[ncols];
    std::vector<int> lay_col(L, -1);
    for (int c = 0; c < ncols; ++c)
        for (int l = off[c]; l < end[c]; ++l) lay_col[l] = c;
    const size_t ni = h->ni;
    cudaStream_t s = h->stream;
    VK_CUDA(h, cudaMemcpyAsync(h->d_col_off, off.data(), off.size() * sizeof(int), cudaMemcpyHostToDevice, s));
    VK_CUDA(h, cudaMemcpyAsync(h->d_col_end, end.data(), end.size() * sizeof(int), cudaMemcpyHostToDevice, s));
    VK_CUDA(h, cudaMemcpyAsync(h->d_lay_col, lay_col.data(), L * sizeof(int), cudaMemcpyHostToDevice, s));
    if (slot_cap) {
        // gap layers hold zeros (finite) in every per-layer input
        VK_CUDA(h, cudaMemsetAsync(h->d_k, 0, (size_t)L * h->nr * sizeof(double), s));
        VK_CUDA(h, cudaMemsetAsync(h->d_atm, 0, (size_t)L * VK_ATM_NF * sizeof(double), s));
        VK_CUDA(h, cudaMemsetAsync(h->d_Dzz, 0, (size_t)L * ni * sizeof(double), s));
        VK_CUDA(h, cudaMemsetAsync(h->w.y, 0, (size_t)L * ni * sizeof(double), s));
        VK_CUDA(h, cudaMemsetAsync(h->w.ymix, 0, (size_t)L * ni * sizeof(double), s));
    }
    // per column (one copy per array when packed: the ranges are contiguous)
    const int nblk = slot_cap ? ncols : 1;
    for (int c = 0; c < nblk; ++c) {
        const int src = slot_cap ? pk[c] : 0, dst = off[c], n = slot_cap ? nz[c] : L;
        VK_CUDA(h, cudaMemcpyAsync(h->d_k + (size_t)dst * h->nr, k + (size_t)src * h->nr,
                                   (size_t)n * h->nr * sizeof(double), cudaMemcpyHostToDevice, s));
        VK_CUDA(h, cudaMemcpyAsync(h->d_atm + (size_t)dst * VK_ATM_NF, atm + (size_t)src * VK_ATM_NF,
                                   (size_t)n * VK_ATM_NF * sizeof(double), cudaMemcpyHostToDevice, s));
        VK_CUDA(h, cudaMemcpyAsync(h->d_Dzz + (size_t)dst * ni, Dzz + (size_t)src * ni,
                                   (size_t)n * ni * sizeof(double), cudaMemcpyHostToDevice, s));
        VK_CUDA(h, cudaMemcpyAsync(h->w.y + (size_t)dst * ni, y + (size_t)src * ni,
                                   (size_t)n * ni * sizeof(double), cudaMemcpyHostToDevice, s));
        VK_CUDA(h, cudaMemcpyAsync(h->w.ymix + (size_t)dst * ni, ymix + (size_t)src * ni,
                                   (size_t)n * ni * sizeof(double), cudaMemcpyHostToDevice, s));
    }
    VK_CUDA(h, cudaMemcpyAsync(h->d_spf, spf, (size_t)ncols * VK_SP_NF * ni * sizeof(double), cudaMemcpyHostToDevice, s));
    VK_CUDA(h, cudaStreamSynchronize(s));
    if (h->ncols != ncols || h->L != L) drop_graph(h);
    h->ncols = ncols;
    h->L = L;
    h->col_off = off;
    h->col_end = end;
    h->slot_cap = slot_cap;
    h->geo_flags = -1;
    int rc = upload_order(h);
    if (rc) return rc;
    VK_CUDA(h, cudaMemset(h->rs.pref, 0, ncols * sizeof(int)));
    std::vector<int> all(ncols);
    for (int c = 0; c < ncols; ++c) all[c] = c;
    return reset_columns(h, all);
}

extern "C" int vk_set_columns(vk_handle *h, int ncols, const int *nz, const double *k,
                              const double *atm, const double *Dzz, const double *spf,
                              const double *y, const double *ymix) {
    return set_columns_impl(h, ncols, 0, nz, k, atm, Dzz, spf, y, ymix);
}

extern "C" int vk_set_columns_slotted(vk_handle *h, int ncols, int slot_cap, const int *nz,
                                      const double *k, const double *atm, const double *Dzz,
                                      const double *spf, const double *y, const double *ymix) {
    if (slot_cap < 2) return fail(h, VK_EINVAL, "slot_cap must be at least 2");
    return set_columns_impl(h, ncols, slot_cap, nz, k, atm, Dzz, spf, y, ymix);
}

extern "C" int vk_refill(vk_handle *h, int n, const int *slots, const int *nz, const double *k,
                         const double *atm, const double *Dzz, const double *spf, const double *y,
                         const double *ymix, const double *atom_ini, const int *pref_indx,
                         const int *conv_ignore) {
    if (!h) return fail(nullptr, VK_EINVAL, "handle is NULL");
    if (!h->slot_cap) return fail(h, VK_EINVAL, "refill needs the slotted layout (vk_set_columns_slotted)");
    if (n <= 0) return VK_OK;
    if (!slots || !nz || !k || !atm || !Dzz || !spf || !y || !ymix || !atom_ini || !pref_indx)
        return fail(h, VK_EINVAL, "NULL input array");
    const size_t ni = h->ni;
    std::vector<int> seen(h->ncols, 0);
    for (int i = 0; i < n; ++i) {
        const int c = slots[i];
        if (c < 0 || c >= h->ncols || seen[c]++) return fail(h, VK_EINVAL, "bad or repeated slot");
        if (nz[i] < 2 || nz[i] > h->slot_cap) return fail(h, VK_EINVAL, "refill column exceeds slot_cap");
        if (pref_indx[i] < 0 || pref_indx[i] >= nz[i]) return fail(h, VK_EINVAL, "pref_indx outside the column");
    }
    cudaStream_t s = h->stream;
    VK_CUDA(h, cudaStreamSynchronize(s));
    size_t src = 0;
    std::vector<int> lay(h->slot_cap);
    for (int i = 0; i < n; ++i) {
        const int c = slots[i], dst = h->col_off[c];
        const size_t m = nz[i];
        VK_CUDA(h, cudaMemcpyAsync(h->d_k + (size_t)dst * h->nr, k + src * h->nr, m * h->nr * sizeof(double), cudaMemcpyHostToDevice, s));
        VK_CUDA(h, cudaMemcpyAsync(h->d_atm + (size_t)dst * VK_ATM_NF, atm + src * VK_ATM_NF, m * VK_ATM_NF * sizeof(double), cudaMemcpyHostToDevice, s));
        VK_CUDA(h, cudaMemcpyAsync(h->d_Dzz + (size_t)dst * ni, Dzz + src * ni, m * ni * sizeof(double), cudaMemcpyHostToDevice, s));
        VK_CUDA(h, cudaMemcpyAsync(h->w.y + (size_t)dst * ni, y + src * ni, m * ni * sizeof(double), cudaMemcpyHostToDevice, s));
        VK_CUDA(h, cudaMemcpyAsync(h->w.ymix + (size_t)dst * ni, ymix + src * ni, m * ni * sizeof(double), cudaMemcpyHostToDevice, s));
        VK_CUDA(h, cudaMemcpyAsync(h->d_spf + (size_t)c * VK_SP_NF * ni, spf + (size_t)i * VK_SP_NF * ni, VK_SP_NF * ni * sizeof(double), cudaMemcpyHostToDevice, s));
        VK_CUDA(h, cudaMemcpyAsync(h->rs.atom_ini + (size_t)c * VK_MAX_NATOM, atom_ini + (size_t)i * h->natom, h->natom * sizeof(double), cudaMemcpyHostToDevice, s));
        VK_CUDA(h, cudaMemcpyAsync(h->rs.pref + c, pref_indx + i, sizeof(int), cudaMemcpyHostToDevice, s));
        if (conv_ignore)
            VK_CUDA(h, cudaMemcpyAsync(h->rs.ignore + (size_t)c * ni, conv_ignore + (size_t)i * ni, ni * sizeof(int), cudaMemcpyHostToDevice, s));
        for (int l = 0; l < h->slot_cap; ++l) lay[l] = l < (int)m ? c : -1;
        VK_CUDA(h, cudaMemcpyAsync(h->d_lay_col + dst, lay.data(), h->slot_cap * sizeof(int), cudaMemcpyHostToDevice, s));
        VK_CUDA(h, cudaStreamSynchronize(s));   // lay is reused
        h->col_end[c] = dst + (int)m;
        src += m;
    }
    VK_CUDA(h, cudaMemcpyAsync(h->d_col_end, h->col_end.data(), h->ncols * sizeof(int), cudaMemcpyHostToDevice, s));
    VK_CUDA(h, cudaStreamSynchronize(s));
    h->geo_flags = -1;                            // transport geometry of the new columns
    int rc = upload_order(h);
    if (rc) return rc;
    std::vector<int> cs(slots, slots + n);
    return reset_columns(h, cs);
}

static int need_batch(vk_handle *h) {
    if (!h) return fail(nullptr, VK_EINVAL, "handle is NULL");
    if (h->ncols == 0) return fail(h, VK_EINVAL, "no columns loaded (call vk_set_columns)");
    return VK_OK;
}

extern "C" int vk_update_state(vk_handle *h, const double *y, const double *ymix) {
    int rc = need_batch(h);
    if (rc) return rc;
    size_t bytes = (size_t)h->L * h->ni * sizeof(double);
    if (y) VK_CUDA(h, cudaMemcpyAsync(h->w.y, y, bytes, cudaMemcpyHostToDevice, h->stream));
    if (ymix) VK_CUDA(h, cudaMemcpyAsync(h->w.ymix, ymix, bytes, cudaMemcpyHostToDevice, h->stream));
    VK_CUDA(h, cudaStreamSynchronize(h->stream));
    return VK_OK;
}

extern "C" int vk_update_atm(vk_handle *h, const double *atm) {
    int rc = need_batch(h);
    if (rc) return rc;
    if (!atm) return fail(h, VK_EINVAL, "atm is NULL");
    VK_CUDA(h, cudaMemcpyAsync(h->d_atm, atm, (size_t)h->L * VK_ATM_NF * sizeof(double),
                               cudaMemcpyHostToDevice, h->stream));
    VK_CUDA(h, cudaStreamSynchronize(h->stream));
    h->geo_flags = -1;
    return VK_OK;
}

extern "C" int vk_update_k(vk_handle *h, const double *k) {
    int rc = need_batch(h);
    if (rc) return rc;
    if (!k) return fail(h, VK_EINVAL, "k is NULL");
    VK_CUDA(h, cudaMemcpyAsync(h->d_k, k, (size_t)h->L * h->nr * sizeof(double),
                               cudaMemcpyHostToDevice, h->stream));
    VK_CUDA(h, cudaStreamSynchronize(h->stream));
    return VK_OK;
}

// Transport geometry for the current atmosphere (recomputed only when the
// atmosphere or the transport flags changed).
static void ensure_geometry(vk_handle *h, int flags) {
    if (h->geo_flags == flags) return;
    vk::launch_geometry(h->net(), h->batch(), h->w.geo, flags, h->stream);
    h->geo_flags = flags;
}

// Enqueue the kernels of one Ros2 attempt for the columns b.active selects
// (all when NULL): device state in, w.sol / w.ymix_out / w.delta out.
static void enqueue_attempt_kernels(vk_handle *h, const DevNet &net, const DevBatch &b, int flags,
                                    double mtol, double atol, bool timed) {
    vk::Work &w = h->w;
    cudaStream_t s = h->stream;
    if (timed) cudaEventRecord(h->ev[0], s);
    vk::launch_rates(net, b, w.y, w.f, w.jv, w.dA, w.dB, w.dC, nullptr, w.dt, w.geo, flags, true, s);
    if (timed) cudaEventRecord(h->ev[1], s);
    if (h->precision == VK_PREC_FP64) {
        vk::launch_lu_fwd_f64(net, b, w, w.f, w.z, flags, s);
        if (timed) cudaEventRecord(h->ev[2], s);
        vk::launch_back_f64(net, b, w.G, w.dB, w.z, w.k1, w.y, w.yk2, w.status, s);
        vk::launch_rates(net, b, w.yk2, w.f, nullptr, nullptr, nullptr, nullptr, w.k1, w.dt, w.geo, flags, false, s);
        vk::launch_solve_f64(net, b, w.G, w.dB, w.dC, w.f, w.z, w.k2, w.status, s);
        h->launches += 6;
    } else {
        // route: fallback[c] = column goes to FP64 this attempt, act32[c] = mixed
        cudaMemsetAsync(w.sweeps, 0, sizeof(int), s);
        cudaMemsetAsync(w.refine_err, 0, b.ncols * sizeof(double), s);
        vk::launch_route(b, w, s);
        // the routed columns' FP64 solves run beside the mixed ones, on the
        // second stream with their own work queue (disjoint columns; f(y) and
        // the LHS of the first launch are in place for both)
        cudaStream_t s2 = h->stream2;
        cudaEventRecord(h->ev_fork, s);
        cudaStreamWaitEvent(s2, h->ev_fork, 0);
        DevBatch br = b;
        br.active = w.routed;
        br.queue = h->d_queue2;
        vk::launch_lu_fwd_f64(net, br, w, w.f, w.z, flags, s2);
        vk::launch_back_f64(net, br, w.G, w.dB, w.z, w.k1, w.y, w.yk2, w.status, s2);
        vk::launch_rates(net, br, w.yk2, w.f, nullptr, nullptr, nullptr, nullptr, w.k1, w.dt, w.geo, flags, false, s2);
        vk::launch_solve_f64(net, br, w.G, w.dB, w.dC, w.f, w.z, w.k2, w.status, s2);
        cudaEventRecord(h->ev_join, s2);
        DevBatch b32 = b;
        b32.active = w.act32;
        vk::launch_lu_reg32(net, b32, w, s);
        if (timed) cudaEventRecord(h->ev[2], s);
        vk::launch_refine(net, b32, w, w.f, w.k1, w.y, w.yk2, h->max_refine, h->refine_tol, s);
        vk::launch_rates(net, b32, w.yk2, w.f2, nullptr, nullptr, nullptr, nullptr, w.k1, w.dt, w.geo, flags, false, s);
        vk::launch_refine(net, b32, w, w.f2, w.k2, w.y, nullptr, h->max_refine, h->refine_tol, s);
        cudaStreamWaitEvent(s, h->ev_join, 0);
        // columns whose refinement failed: FP64 after the others (their f(y)
        // is still in place: neither branch wrote it)
        DevBatch bf = b;
        bf.active = w.failed;
        vk::launch_lu_fwd_f64(net, bf, w, w.f, w.z, flags, s);
        vk::launch_back_f64(net, bf, w.G, w.dB, w.z, w.k1, w.y, w.yk2, w.status, s);
        vk::launch_rates(net, bf, w.yk2, w.f, nullptr, nullptr, nullptr, nullptr, w.k1, w.dt, w.geo, flags, false, s);
        vk::launch_solve_f64(net, bf, w.G, w.dB, w.dC, w.f, w.z, w.k2, w.status, s);
        h->launches += 16;
    }
    if (timed) cudaEventRecord(h->ev[3], s);
    vk::launch_stage(net, b, w, flags, mtol, atol, s);
    if (timed) cudaEventRecord(h->ev[4], s);
}

static int enqueue_attempt(vk_handle *h, int flags, bool timed) {
    if (h->precision == VK_PREC_MIXED && !h->w.G32)
        return fail(h, VK_EINVAL, "mixed precision not allocated on this handle");
    ensure_geometry(h, flags);
    enqueue_attempt_kernels(h, h->net(), h->batch(), flags, 1.E-22, 1.E-1, timed);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(h, VK_ECUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
    return VK_OK;
}

extern "C" int vk_ros2_attempt(vk_handle *h, const double *dt, int flags, double *sol,
                               double *ymix, double *delta, double *k1, double *k2) {
    int rc = need_batch(h);
    if (rc) return rc;
    if (!dt) return fail(h, VK_EINVAL, "dt is NULL");
    for (int c = 0; c < h->ncols; ++c)
        if (!(dt[c] > 0.0) || !std::isfinite(dt[c]))
            return fail(h, VK_EINVAL, "dt must be positive and finite");
    cudaStream_t s = h->stream;
    VK_CUDA(h, cudaMemcpyAsync(h->w.dt, dt, h->ncols * sizeof(double), cudaMemcpyHostToDevice, s));
    VK_CUDA(h, cudaMemsetAsync(h->w.status, 0, h->ncols * sizeof(int), s));
    h->launches = 0;
    rc = enqueue_attempt(h, flags, true);
    if (rc) return rc;
    size_t bytes = (size_t)h->L * h->ni * sizeof(double);
    if (sol) VK_CUDA(h, cudaMemcpyAsync(sol, h->w.sol, bytes, cudaMemcpyDeviceToHost, s));
    if (ymix) VK_CUDA(h, cudaMemcpyAsync(ymix, h->w.ymix_out, bytes, cudaMemcpyDeviceToHost, s));
    if (k1) VK_CUDA(h, cudaMemcpyAsync(k1, h->w.k1, bytes, cudaMemcpyDeviceToHost, s));
    if (k2) VK_CUDA(h, cudaMemcpyAsync(k2, h->w.k2, bytes, cudaMemcpyDeviceToHost, s));
    if (delta) VK_CUDA(h, cudaMemcpyAsync(delta, h->w.delta, h->ncols * sizeof(double), cudaMemcpyDeviceToHost, s));
    std::vector<int> st(h->ncols);
    VK_CUDA(h, cudaMemcpyAsync(st.data(), h->w.status, h->ncols * sizeof(int), cudaMemcpyDeviceToHost, s));
    VK_CUDA(h, cudaStreamSynchronize(s));
    cudaEventElapsedTime(&h->ms[0], h->ev[0], h->ev[1]);
    cudaEventElapsedTime(&h->ms[1], h->ev[1], h->ev[2]);
    cudaEventElapsedTime(&h->ms[2], h->ev[2], h->ev[3]);
    cudaEventElapsedTime(&h->ms[3], h->ev[3], h->ev[4]);
    for (int c = 0; c < h->ncols; ++c) {
        if (st[c] == VK_ESINGULAR)
            return fail(h, VK_ESINGULAR, "singular diagonal block in column " + std::to_string(c));
        if (st[c] == VK_ENAN)
            return fail(h, VK_ENAN, "non-finite pivot (NaN state) in column " + std::to_string(c));
    }
    return VK_OK;
}

// Right-hand side of the Ros2 system at state y (or the handle's state when y
// is NULL): chemistry plus the transport terms the flags select, the f of
// op.py:2888 (chemdf + diffdf).
extern "C" int vk_rhs(vk_handle *h, const double *y, int flags, double *f) {
    int rc = need_batch(h);
    if (rc) return rc;
    if (!f) return fail(h, VK_EINVAL, "f is NULL");
    size_t bytes = (size_t)h->L * h->ni * sizeof(double);
    const double *yd = h->w.y;
    if (y) {
        VK_CUDA(h, cudaMemcpyAsync(h->w.yk2, y, bytes, cudaMemcpyHostToDevice, h->stream));
        yd = h->w.yk2;
    }
    ensure_geometry(h, flags);
    vk::launch_rates(h->net(), h->batch(), yd, h->w.f2, h->w.jv, h->w.dA, h->w.dB, h->w.dC, nullptr,
                     h->w.dt, h->w.geo, flags, false, h->stream);
    VK_CUDA(h, cudaGetLastError());
    VK_CUDA(h, cudaMemcpyAsync(f, h->w.f2, bytes, cudaMemcpyDeviceToHost, h->stream));
    VK_CUDA(h, cudaStreamSynchronize(h->stream));
    return VK_OK;
}

// Test hook: chemistry source term only (the generated chemdf) of the state y.
extern "C" int vk_chem_source(vk_handle *h, const double *y, double *dydt) {
    int rc = need_batch(h);
    if (rc) return rc;
    size_t bytes = (size_t)h->L * h->ni * sizeof(double);
    if (y) VK_CUDA(h, cudaMemcpyAsync(h->w.y, y, bytes, cudaMemcpyHostToDevice, h->stream));
    ensure_geometry(h, 0);
    vk::launch_chem_only(h->net(), h->batch(), h->w.y, h->w.f, h->w.geo, h->stream);
    VK_CUDA(h, cudaGetLastError());
    VK_CUDA(h, cudaMemcpyAsync(dydt, h->w.f, bytes, cudaMemcpyDeviceToHost, h->stream));
    VK_CUDA(h, cudaStreamSynchronize(h->stream));
    return VK_OK;
}

// Test hook: the LHS pieces of the last attempt (-J entries, diffusion coefficients).
extern "C" int vk_get_lhs(vk_handle *h, double *jv, double *dA, double *dB, double *dC) {
    int rc = need_batch(h);
    if (rc) return rc;
    size_t nb = (size_t)h->L * h->ni * sizeof(double);
    if (jv) VK_CUDA(h, cudaMemcpy(jv, h->w.jv, (size_t)h->L * h->nnz * sizeof(double), cudaMemcpyDeviceToHost));
    if (dA) VK_CUDA(h, cudaMemcpy(dA, h->w.dA, nb, cudaMemcpyDeviceToHost));
    if (dB) VK_CUDA(h, cudaMemcpy(dB, h->w.dB, nb, cudaMemcpyDeviceToHost));
    if (dC) VK_CUDA(h, cudaMemcpy(dC, h->w.dC, nb, cudaMemcpyDeviceToHost));
    return VK_OK;
}

// Test hook: the FP32 inverses of the scaled blocks of the last mixed attempt,
// [L][ni*ni] natural order (layers of columns solved in FP64 are stale).
extern "C" int vk_get_lu32(vk_handle *h, float *G) {
    int rc = need_batch(h);
    if (rc) return rc;
    if (!G) return fail(h, VK_EINVAL, "G is NULL");
    if (!h->w.G32) return fail(h, VK_EINVAL, "no FP32 factors (precision is FP64)");
    const size_t nn = (size_t)h->ni * h->ni, st = (nn + 3) & ~(size_t)3;
    VK_CUDA(h, cudaStreamSynchronize(h->stream));
    VK_CUDA(h, cudaMemcpy2D(G, nn * sizeof(float), h->w.G32, st * sizeof(float), nn * sizeof(float),
                            h->L, cudaMemcpyDeviceToHost));
    return VK_OK;
}

extern "C" int vk_get_timing(vk_handle *h, double *ms_rates, double *ms_lu, double *ms_solve,
                             double *ms_stage, int *launches) {
    if (!h) return fail(nullptr, VK_EINVAL, "handle is NULL");
    if (ms_rates) *ms_rates = h->ms[0];
    if (ms_lu) *ms_lu = h->ms[1];
    if (ms_solve) *ms_solve = h->ms[2];
    if (ms_stage) *ms_stage = h->ms[3];
    if (launches) *launches = h->launches;
    return VK_OK;
}

extern "C" int vk_set_atom_ini(vk_handle *h, const double *atom_ini) {
    int rc = need_batch(h);
    if (rc) return rc;
    if (!atom_ini) return fail(h, VK_EINVAL, "atom_ini is NULL");
    std::vector<double> buf((size_t)h->ncols * VK_MAX_NATOM, 0.0);
    for (int c = 0; c < h->ncols; ++c)
        for (int a = 0; a < h->natom; ++a) buf[(size_t)c * VK_MAX_NATOM + a] = atom_ini[(size_t)c * h->natom + a];
    VK_CUDA(h, cudaMemcpy(h->rs.atom_ini, buf.data(), buf.size() * sizeof(double), cudaMemcpyHostToDevice));
    return VK_OK;
}

extern "C" int vk_set_column_info(vk_handle *h, const int *pref_indx, const int *conv_ignore) {
    int rc = need_batch(h);
    if (rc) return rc;
    if (pref_indx) {
        for (int c = 0; c < h->ncols; ++c)
            if (pref_indx[c] < 0 || pref_indx[c] >= h->col_end[c] - h->col_off[c])
                return fail(h, VK_EINVAL, "pref_indx outside the column");
        VK_CUDA(h, cudaMemcpy(h->rs.pref, pref_indx, h->ncols * sizeof(int), cudaMemcpyHostToDevice));
    }
    if (conv_ignore) {                    // one mask for every column
        std::vector<int> m((size_t)h->ncols * h->ni);
        for (int c = 0; c < h->ncols; ++c)
            std::copy(conv_ignore, conv_ignore + h->ni, m.begin() + (size_t)c * h->ni);
        VK_CUDA(h, cudaMemcpy(h->rs.ignore, m.data(), m.size() * sizeof(int), cudaMemcpyHostToDevice));
    }
    return VK_OK;
}

extern "C" int vk_set_conv_ignore(vk_handle *h, const int *conv_ignore) {
    int rc = need_batch(h);
    if (rc) return rc;
    if (!conv_ignore) return fail(h, VK_EINVAL, "conv_ignore is NULL");
    VK_CUDA(h, cudaMemcpy(h->rs.ignore, conv_ignore, (size_t)h->ncols * h->ni * sizeof(int),
                          cudaMemcpyHostToDevice));
    return VK_OK;
}

extern "C" int vk_set_clock(vk_handle *h, const double *dt, const double *t, const int *count) {
    int rc = need_batch(h);
    if (rc) return rc;
    if (dt) VK_CUDA(h, cudaMemcpy(h->w.dt, dt, h->ncols * sizeof(double), cudaMemcpyHostToDevice));
    if (t) VK_CUDA(h, cudaMemcpy(h->rs.t, t, h->ncols * sizeof(double), cudaMemcpyHostToDevice));
    if (count) VK_CUDA(h, cudaMemcpy(h->rs.count, count, h->ncols * sizeof(int), cudaMemcpyHostToDevice));
    return VK_OK;
}

extern "C" int vk_get_state(vk_handle *h, double *y, double *ymix, double *dt, double *t,
                            int *count, int *end_case, double *delta) {
    int rc = need_batch(h);
    if (rc) return rc;
    size_t nb = (size_t)h->L * h->ni * sizeof(double);
    cudaStream_t s = h->stream;
    if (y) VK_CUDA(h, cudaMemcpyAsync(y, h->w.y, nb, cudaMemcpyDeviceToHost, s));
    if (ymix) VK_CUDA(h, cudaMemcpyAsync(ymix, h->w.ymix, nb, cudaMemcpyDeviceToHost, s));
    if (dt) VK_CUDA(h, cudaMemcpyAsync(dt, h->w.dt, h->ncols * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (t) VK_CUDA(h, cudaMemcpyAsync(t, h->rs.t, h->ncols * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (count) VK_CUDA(h, cudaMemcpyAsync(count, h->rs.count, h->ncols * sizeof(int), cudaMemcpyDeviceToHost, s));
    if (end_case) VK_CUDA(h, cudaMemcpyAsync(end_case, h->rs.end_case, h->ncols * sizeof(int), cudaMemcpyDeviceToHost, s));
    if (delta) VK_CUDA(h, cudaMemcpyAsync(delta, h->w.delta, h->ncols * sizeof(double), cudaMemcpyDeviceToHost, s));
    VK_CUDA(h, cudaStreamSynchronize(s));
    return VK_OK;
}

extern "C" int vk_get_counters(vk_handle *h, int *counters) {
    int rc = need_batch(h);
    if (rc) return rc;
    if (!counters) return fail(h, VK_EINVAL, "counters is NULL");
    VK_CUDA(h, cudaMemcpy(counters, h->rs.counters, (size_t)h->ncols * VK_NCOUNTERS * sizeof(int), cudaMemcpyDeviceToHost));
    return VK_OK;
}

extern "C" int vk_set_rate_params(vk_handle *h, const int *kind, const int *rev, const double *params,
                                  const double *nasa9) {
    if (!h) return fail(h, VK_EINVAL, "handle is NULL");
    if (!kind || !rev || !params || !nasa9) return fail(h, VK_EINVAL, "rate parameter array is NULL");
    for (int p = 0; p < h->npair; ++p)
        if (kind[p] < VK_K_NONE || kind[p] > VK_K_SPECIAL_OH_CH3)
            return fail(h, VK_EINVAL, "unknown rate kind for pair " + std::to_string(p));
    if (!h->d_kkind) {
        int rc = dalloc(h, &h->d_kkind, h->npair);
        if (!rc) rc = dalloc(h, &h->d_krev, h->npair);
        if (!rc) rc = dalloc(h, &h->d_kpar, (size_t)h->npair * 6);
        if (!rc) rc = dalloc(h, &h->d_nasa9, (size_t)h->ni * 20);
        if (rc) {                          // the handle frees what was allocated
            h->d_kkind = nullptr;
            return rc;
        }
    }
    VK_CUDA(h, cudaMemcpy(h->d_kkind, kind, h->npair * sizeof(int), cudaMemcpyHostToDevice));
    VK_CUDA(h, cudaMemcpy(h->d_krev, rev, h->npair * sizeof(int), cudaMemcpyHostToDevice));
    VK_CUDA(h, cudaMemcpy(h->d_kpar, params, (size_t)h->npair * 6 * sizeof(double), cudaMemcpyHostToDevice));
    VK_CUDA(h, cudaMemcpy(h->d_nasa9, nasa9, (size_t)h->ni * 20 * sizeof(double), cudaMemcpyHostToDevice));
    return VK_OK;
}

extern "C" int vk_set_launch(vk_handle *h, int kernel, int ctas_per_sm, int variant) {
    if (!h) return fail(h, VK_EINVAL, "handle is NULL");
    if (kernel < 0 || kernel >= VK_TUNE_N) return fail(h, VK_EINVAL, "kernel must be a VK_TUNE_* value");
    if (ctas_per_sm < 0 || ctas_per_sm > 8) return fail(h, VK_EINVAL, "ctas_per_sm must be 0..8");
    if (kernel == VK_TUNE_LU32 && variant != -1 &&
        (vk::lu32_tiling_cap(variant) == 0 || vk::lu32_tiling_cap(variant) < h->ni))
        return fail(h, VK_EINVAL, "k_lu32 tiling " + std::to_string(variant) + " does not cover " +
                                      std::to_string(h->ni) + " species");
    if (h->stream) VK_CUDA(h, cudaStreamSynchronize(h->stream));
    drop_graph(h);                         // the captured loop has the old grids
    h->cps_k[kernel] = ctas_per_sm;
    if (kernel == VK_TUNE_LU32) h->lu32_tiling = variant;
    return VK_OK;
}

extern "C" int vk_get_launch(vk_handle *h, int kernel, int *ctas_per_sm, int *variant) {
    if (!h) return fail(h, VK_EINVAL, "handle is NULL");
    if (kernel < 0 || kernel >= VK_TUNE_N) return fail(h, VK_EINVAL, "kernel must be a VK_TUNE_* value");
    if (ctas_per_sm) *ctas_per_sm = h->cps_k[kernel];
    if (variant) *variant = kernel == VK_TUNE_LU32 ? h->lu32_tiling : -1;
    return VK_OK;
}

extern "C" int vk_set_rate_caps(vk_handle *h, const int *kind, const double *t_max,
                                const double *params) {
    if (!h) return fail(h, VK_EINVAL, "handle is NULL");
    if (!kind) {
        h->caps_on = 0;
        return VK_OK;
    }
    if (!t_max || !params) return fail(h, VK_EINVAL, "t_max or params is NULL");
    for (int p = 0; p < h->npair; ++p)
        if (kind[p] != VK_K_NONE && kind[p] != VK_K_ARRHENIUS && kind[p] != VK_K_FALLOFF)
            return fail(h, VK_EINVAL, "cap kind must be VK_K_NONE, VK_K_ARRHENIUS or VK_K_FALLOFF");
    if (!h->d_capk) {
        int rc = dalloc(h, &h->d_capk, (size_t)h->npair);
        if (!rc) rc = dalloc(h, &h->d_capT, (size_t)h->npair);
        if (!rc) rc = dalloc(h, &h->d_capp, (size_t)h->npair * 6);
        if (rc) {                          // the handle frees what was allocated
            h->d_capk = nullptr;
            return rc;
        }
    }
    VK_CUDA(h, cudaStreamSynchronize(h->stream));
    VK_CUDA(h, cudaMemcpy(h->d_capk, kind, h->npair * sizeof(int), cudaMemcpyHostToDevice));
    VK_CUDA(h, cudaMemcpy(h->d_capT, t_max, h->npair * sizeof(double), cudaMemcpyHostToDevice));
    VK_CUDA(h, cudaMemcpy(h->d_capp, params, (size_t)h->npair * 6 * sizeof(double), cudaMemcpyHostToDevice));
    h->caps_on = 1;
    return VK_OK;
}

extern "C" int vk_photo_setup(vk_handle *h, int nbins, const double *bins, const double *jweights,
                              int nabs, const int *abs_sp, const int *abs_photo, const double *cross,
                              int nscat, const int *scat_sp, const double *cross_scat, int nch,
                              const int *ch_kindex, const double *cross_J, const double *sflux_top,
                              double sl_angle, double edd, double f_diurnal, double flux_atol) {
    if (!h) return fail(h, VK_EINVAL, "handle is NULL");
    if (h->ph.nbins) return fail(h, VK_EINVAL, "radiative transfer already set up on this handle");
    if (nbins < 2 || nabs < 1 || nscat < 0 || nch < 1)
        return fail(h, VK_EINVAL, "need nbins >= 2, nabs >= 1, nscat >= 0, nch >= 1");
    if (!bins || !jweights || !abs_sp || !abs_photo || !cross || !ch_kindex || !cross_J || !sflux_top ||
        (nscat && (!scat_sp || !cross_scat)))
        return fail(h, VK_EINVAL, "radiative-transfer array is NULL");
    for (int a = 0; a < nabs; ++a)
        if (abs_sp[a] < 0 || abs_sp[a] >= h->ni) return fail(h, VK_EINVAL, "absorber species out of range");
    for (int a = 0; a < nscat; ++a)
        if (scat_sp[a] < 0 || scat_sp[a] >= h->ni) return fail(h, VK_EINVAL, "scatterer species out of range");
    for (int c = 0; c < nch; ++c)
        if (ch_kindex[c] < 1 || ch_kindex[c] > h->nr) return fail(h, VK_EINVAL, "channel k index out of range");
    if (!(edd > 0) || !(cos(sl_angle) > 0)) return fail(h, VK_EINVAL, "need edd > 0 and cos(sl_angle) > 0");
    std::vector<double> wcj((size_t)nch * nbins);
    for (int c = 0; c < nch; ++c)
        for (int n = 0; n < nbins; ++n) wcj[(size_t)c * nbins + n] = cross_J[(size_t)c * nbins + n] * jweights[n];
    PhotoDev &p = h->ph;
    const size_t st = (size_t)(h->max_layers + h->max_cols) * nbins, ly = (size_t)h->max_layers * nbins;
    int rc = 0;
    double *db = nullptr, *dc = nullptr, *dsc = nullptr, *dw = nullptr, *dtop = nullptr;
    int *das = nullptr, *dap = nullptr, *dss = nullptr, *dki = nullptr;
    std::vector<double> bv(bins, bins + nbins), cv(cross, cross + (size_t)nabs * nbins),
        topv(sflux_top, sflux_top + nbins), scv;
    std::vector<int> asv(abs_sp, abs_sp + nabs), apv(abs_photo, abs_photo + nabs),
        kiv(ch_kindex, ch_kindex + nch), ssv;
    if (nscat) {
        scv.assign(cross_scat, cross_scat + (size_t)nscat * nbins);
        ssv.assign(scat_sp, scat_sp + nscat);
    }
    if (!rc) rc = upload(h, &db, bv);
    if (!rc) rc = upload(h, &dc, cv);
    if (!rc) rc = upload(h, &dsc, scv);
    if (!rc) rc = upload(h, &dw, wcj);
    if (!rc) rc = upload(h, &dtop, topv);
    if (!rc) rc = upload(h, &das, asv);
    if (!rc) rc = upload(h, &dap, apv);
    if (!rc) rc = upload(h, &dss, ssv);
    if (!rc) rc = upload(h, &dki, kiv);
    double **big[] = {&p.tau, &p.dflux_u, &p.dflux_d};
    for (double **q : big) if (!rc) rc = dalloc(h, q, st);
    double **lay[] = {&p.w0, &p.aflux, &p.aflux_prev};
    for (double **q : lay) if (!rc) rc = dalloc(h, q, ly);
    if (!rc) rc = dalloc(h, &p.J, (size_t)h->max_layers * nch);
    if (!rc) rc = dalloc(h, &h->d_phmask, h->max_cols);
    if (rc) return rc;                     // the handle frees what was allocated
    p.bins = db; p.cross = dc; p.cross_scat = dsc; p.wcross_J = dw; p.sflux_top = dtop;
    p.abs_sp = das; p.abs_photo = dap; p.scat_sp = dss; p.ch_kindex = dki;
    p.nabs = nabs; p.nscat = nscat; p.nch = nch;
    p.abs_tslot = nullptr; p.cross_T = nullptr; p.ch_tslot = nullptr; p.wcross_J_T = nullptr;
    p.lstride = h->max_layers;
    h->ph_jw.assign(jweights, jweights + nbins);
    p.sl_angle = sl_angle; p.edd = edd; p.f_diurnal = f_diurnal; p.flux_atol = flux_atol;
    VK_CUDA(h, cudaMemset(p.dflux_u, 0, st * sizeof(double)));
    VK_CUDA(h, cudaMemset(p.dflux_d, 0, st * sizeof(double)));
    VK_CUDA(h, cudaMemset(p.aflux, 0, ly * sizeof(double)));
    p.nbins = nbins;
    return VK_OK;
}

extern "C" int vk_photo_set_cross_T(vk_handle *h, int nabs_t, const int *abs_slot,
                                    const double *cross_T, int nch_t, const int *ch_slot,
                                    const double *cross_J_T) {
    int rc = need_batch(h);
    if (rc) return rc;
    PhotoDev &p = h->ph;
    if (!p.nbins) return fail(h, VK_EINVAL, "no radiative transfer (call vk_photo_setup)");
    if (nabs_t < 0 || nabs_t > p.nabs || nch_t < 0 || nch_t > p.nch)
        return fail(h, VK_EINVAL, "nabs_t / nch_t out of range");
    if ((nabs_t && (!abs_slot || !cross_T)) || (nch_t && (!ch_slot || !cross_J_T)))
        return fail(h, VK_EINVAL, "T-dependent cross-section array is NULL");
    std::vector<int> at(p.nabs, -1), ct(p.nch, -1);
    for (int i = 0; i < nabs_t; ++i) {
        if (abs_slot[i] < 0 || abs_slot[i] >= p.nabs || at[abs_slot[i]] >= 0)
            return fail(h, VK_EINVAL, "absorber slot out of range or repeated");
        at[abs_slot[i]] = i;
    }
    for (int i = 0; i < nch_t; ++i) {
        if (ch_slot[i] < 0 || ch_slot[i] >= p.nch || ct[ch_slot[i]] >= 0)
            return fail(h, VK_EINVAL, "channel slot out of range or repeated");
        ct[ch_slot[i]] = i;
    }
    VK_CUDA(h, cudaStreamSynchronize(h->stream));   // no update reads the tables meanwhile
    p.abs_tslot = nullptr; p.cross_T = nullptr; p.ch_tslot = nullptr; p.wcross_J_T = nullptr;
    if (!nabs_t && !nch_t) return VK_OK;
    const size_t NB = (size_t)p.nbins, LS = (size_t)h->max_layers, L = (size_t)h->L;
    if (!h->d_abs_tslot) {
        rc = dalloc(h, &h->d_abs_tslot, (size_t)p.nabs);
        if (!rc) rc = dalloc(h, &h->d_ch_tslot, (size_t)p.nch);
        if (rc) return rc;
    }
    if (nabs_t > h->tcap_abs) {
        dfree(h, h->d_crossT);
        h->d_crossT = nullptr;
        h->tcap_abs = 0;
        if ((rc = dalloc(h, &h->d_crossT, (size_t)nabs_t * LS * NB))) return rc;
        h->tcap_abs = nabs_t;
    }
    if (nch_t > h->tcap_ch) {
        dfree(h, h->d_wcrossJT);
        h->d_wcrossJT = nullptr;
        h->tcap_ch = 0;
        if ((rc = dalloc(h, &h->d_wcrossJT, (size_t)nch_t * LS * NB))) return rc;
        h->tcap_ch = nch_t;
    }
    VK_CUDA(h, cudaMemcpy(h->d_abs_tslot, at.data(), at.size() * sizeof(int), cudaMemcpyHostToDevice));
    VK_CUDA(h, cudaMemcpy(h->d_ch_tslot, ct.data(), ct.size() * sizeof(int), cudaMemcpyHostToDevice));
    for (int i = 0; i < nabs_t; ++i)
        VK_CUDA(h, cudaMemcpy(h->d_crossT + i * LS * NB, cross_T + i * L * NB, L * NB * sizeof(double),
                              cudaMemcpyHostToDevice));
    std::vector<double> w(L * NB);
    for (int i = 0; i < nch_t; ++i) {
        const double *src = cross_J_T + i * L * NB;
        for (size_t l = 0; l < L; ++l)
            for (size_t n = 0; n < NB; ++n) w[l * NB + n] = src[l * NB + n] * h->ph_jw[n];
        VK_CUDA(h, cudaMemcpy(h->d_wcrossJT + i * LS * NB, w.data(), L * NB * sizeof(double),
                              cudaMemcpyHostToDevice));
    }
    p.abs_tslot = h->d_abs_tslot; p.cross_T = h->d_crossT;
    p.ch_tslot = h->d_ch_tslot; p.wcross_J_T = h->d_wcrossJT;
    p.lstride = (int)LS;
    return VK_OK;
}

extern "C" int vk_photo_reset(vk_handle *h) {
    if (!h) return fail(h, VK_EINVAL, "handle is NULL");
    PhotoDev &p = h->ph;
    if (!p.nbins) return fail(h, VK_EINVAL, "no radiative transfer (call vk_photo_setup)");
    const size_t st = (size_t)(h->max_layers + h->max_cols) * p.nbins, ly = (size_t)h->max_layers * p.nbins;
    VK_CUDA(h, cudaMemset(p.dflux_u, 0, st * sizeof(double)));
    VK_CUDA(h, cudaMemset(p.dflux_d, 0, st * sizeof(double)));
    VK_CUDA(h, cudaMemset(p.aflux, 0, ly * sizeof(double)));
    return VK_OK;
}

extern "C" int vk_photo_update(vk_handle *h, const int *col_mask, double *aflux_change) {
    int rc = need_batch(h);
    if (rc) return rc;
    PhotoDev &p = h->ph;
    if (!p.nbins) return fail(h, VK_EINVAL, "no radiative transfer (call vk_photo_setup)");
    cudaStream_t s = h->stream;
    DevBatch b = h->batch();
    if (col_mask) {
        VK_CUDA(h, cudaMemcpyAsync(h->d_phmask, col_mask, h->ncols * sizeof(int), cudaMemcpyHostToDevice, s));
        b.active = h->d_phmask;
    }
    // the change is accumulated as the bit pattern of a non-negative double
    unsigned long long *chg = reinterpret_cast<unsigned long long *>(h->rs.aflux_change);
    vk::launch_photo_clear(b, chg, s);
    vk::launch_photo(h->net(), b, p, h->w.y, h->w.ymix, h->d_k, chg, s);
    VK_CUDA(h, cudaGetLastError());
    if (aflux_change)
        VK_CUDA(h, cudaMemcpyAsync(aflux_change, h->rs.aflux_change, h->ncols * sizeof(double),
                                   cudaMemcpyDeviceToHost, s));
    VK_CUDA(h, cudaStreamSynchronize(s));
    return VK_OK;
}

extern "C" int vk_photo_get(vk_handle *h, double *tau, double *aflux, double *J) {
    int rc = need_batch(h);
    if (rc) return rc;
    PhotoDev &p = h->ph;
    if (!p.nbins) return fail(h, VK_EINVAL, "no radiative transfer (call vk_photo_setup)");
    if (tau) VK_CUDA(h, cudaMemcpy(tau, p.tau, (size_t)(h->L + h->ncols) * p.nbins * sizeof(double), cudaMemcpyDeviceToHost));
    if (aflux) VK_CUDA(h, cudaMemcpy(aflux, p.aflux, (size_t)h->L * p.nbins * sizeof(double), cudaMemcpyDeviceToHost));
    if (J) VK_CUDA(h, cudaMemcpy(J, p.J, (size_t)h->L * p.nch * sizeof(double), cudaMemcpyDeviceToHost));
    return VK_OK;
}

extern "C" int vk_compute_k(vk_handle *h) {
    int rc = need_batch(h);
    if (rc) return rc;
    if (!h->d_kkind) return fail(h, VK_EINVAL, "no rate parameters (call vk_set_rate_params)");
    vk::launch_rate_consts(h->net(), h->batch(), h->d_kkind, h->d_krev,
                           h->caps_on ? h->d_capk : nullptr, h->d_capT, h->d_capp, h->d_kpar,
                           h->d_nasa9, h->d_k, h->stream);
    VK_CUDA(h, cudaGetLastError());
    VK_CUDA(h, cudaStreamSynchronize(h->stream));
    return VK_OK;
}

extern "C" int vk_get_k(vk_handle *h, double *k) {
    int rc = need_batch(h);
    if (rc) return rc;
    if (!k) return fail(h, VK_EINVAL, "k is NULL");
    VK_CUDA(h, cudaMemcpy(k, h->d_k, (size_t)h->L * h->nr * sizeof(double), cudaMemcpyDeviceToHost));
    return VK_OK;
}

// Diagnostic: the last steady-state test's longdy and longdydt per column
// (Integration.conv, op.py:1046-1049); zero before a column's first test.
extern "C" int vk_get_conv(vk_handle *h, double *longdy, double *longdydt) {
    int rc = need_batch(h);
    if (rc) return rc;
    if (longdy) VK_CUDA(h, cudaMemcpy(longdy, h->rs.longdy, h->ncols * sizeof(double), cudaMemcpyDeviceToHost));
    if (longdydt) VK_CUDA(h, cudaMemcpy(longdydt, h->rs.longdydt, h->ncols * sizeof(double), cudaMemcpyDeviceToHost));
    return VK_OK;
}

static vk::RunCtrl to_run_ctrl(const vk_ctrl *c, int max_steps) {
    vk::RunCtrl r;
    std::memset(&r, 0, sizeof(r));
    r.rtol = c->rtol; r.atol = c->atol; r.mtol = c->mtol; r.mtol_conv = c->mtol_conv;
    r.pos_cut = c->pos_cut; r.nega_cut = c->nega_cut; r.loss_eps = c->loss_eps;
    r.dt_min = c->dt_min; r.dt_max = c->dt_max; r.dt_var_min = c->dt_var_min; r.dt_var_max = c->dt_var_max;
    r.yconv_cri = c->yconv_cri; r.slope_cri = c->slope_cri; r.yconv_min = c->yconv_min;
    r.st_factor = c->st_factor; r.trun_min = c->trun_min; r.runtime = c->runtime;
    r.gs = c->gs; r.Rp = c->Rp; r.flux_cri = c->flux_cri;
    r.conv_step = c->conv_step; r.count_min = c->count_min; r.count_max = c->count_max;
    r.update_frq = c->update_frq; r.max_attempts = c->max_attempts; r.flags = c->flags;
    r.max_steps = max_steps > 0 ? max_steps : INT_MAX;
    return r;
}

static const int kGraphAttempts = 8;

// Attempts per replay of the run loop: a call of fewer steps than
// kGraphAttempts (one step per call is the reference's own pattern) replays
// that many, so the attempts after every column has taken its steps are not
// launched; a rejection costs one more replay.
static int graph_attempts(const vk::RunCtrl &cc) {
    return cc.max_steps < kGraphAttempts ? cc.max_steps : kGraphAttempts;
}

// Everything of a run before its replays, on h->stream: the control values'
// check, the history ring (conv_step accepted states of the whole batch),
// the transport geometry and the per-call start of every column.
static int run_prepare(vk_handle *h, const vk_ctrl *ctrl, int max_steps, vk::RunCtrl &cc) {
    int rc = need_batch(h);
    if (rc) return rc;
    if (!ctrl) return fail(h, VK_EINVAL, "ctrl is NULL");
    if (ctrl->conv_step < 2 || ctrl->update_frq < 1 || ctrl->max_attempts < 1 || ctrl->rtol <= 0)
        return fail(h, VK_EINVAL, "bad control values");
    cc = to_run_ctrl(ctrl, max_steps);
    cudaStream_t s = h->stream;
    if (h->hist_R != cc.conv_step || !h->rs.hist_y) {
        if (h->rs.hist_y) { cudaFree(h->rs.hist_y); cudaFree(h->rs.hist_t); }
        h->rs.hist_y = nullptr; h->rs.hist_t = nullptr;
        drop_graph(h);
        cudaError_t e1 = cudaMalloc(&h->rs.hist_y, (size_t)cc.conv_step * h->max_layers * h->ni * sizeof(double));
        cudaError_t e2 = cudaMalloc(&h->rs.hist_t, (size_t)cc.conv_step * h->max_cols * sizeof(double));
        if (e1 != cudaSuccess || e2 != cudaSuccess) {
            if (h->rs.hist_y) cudaFree(h->rs.hist_y);
            if (h->rs.hist_t) cudaFree(h->rs.hist_t);
            h->rs.hist_y = nullptr; h->rs.hist_t = nullptr; h->hist_R = 0;
            return fail(h, VK_ENOMEM, "history ring allocation failed");
        }
        h->hist_R = cc.conv_step;
    }
    if (h->precision == VK_PREC_MIXED && !h->w.G32)
        return fail(h, VK_EINVAL, "mixed precision not allocated on this handle");
    ensure_geometry(h, cc.flags);
    DevBatch b = h->batch();
    b.active = h->rs.active;
    VK_CUDA(h, cudaMemsetAsync(h->w.status, 0, h->ncols * sizeof(int), s));
    vk::launch_start(h->net(), b, h->rs, cc, s);
    VK_CUDA(h, cudaGetLastError());
    return VK_OK;
}

// What a captured loop of h depends on besides its buffers (those are
// covered by h->gen): the control values and the batch shape.
static void run_key(const vk_handle *h, const vk::RunCtrl &cc, unsigned char *key) {
    std::memcpy(key, &cc, sizeof(cc));
    std::memcpy(key + sizeof(cc), &h->ncols, sizeof(int));
    std::memcpy(key + sizeof(cc) + sizeof(int), &h->L, sizeof(int));
}

// The replayed body on h->stream: ga attempts, each followed by the control
// step of every active column (accept/reject, dt, steady-state test), then
// the count of the columns still running into h->d_nactive.
static void run_body(vk_handle *h, const vk::RunCtrl &cc, int ga) {
    DevNet net = h->net();
    DevBatch b = h->batch();
    b.active = h->rs.active;
    vk::Work &w = h->w;
    for (int it = 0; it < ga; ++it) {
        enqueue_attempt_kernels(h, net, b, cc.flags, cc.mtol, cc.atol, false);
        vk::launch_control(net, b, h->rs, cc, w.sol, w.ymix_out, w.delta, w.status,
                           h->precision == VK_PREC_MIXED ? w.fallback : nullptr, w.geo, h->stream);
    }
    vk::launch_count_active(h->rs.active, h->ncols, h->d_nactive, h->stream);
}

// Launches of one replay of h's body (the gpu_launches count).
static int body_launches(const vk_handle *h, int ga) {
    return ga * (h->precision == VK_PREC_MIXED ? 17 : 7) + 1;
}

// A column that stopped with an error status fails the call.
static int run_check_end(vk_handle *h) {
    std::vector<int> ec(h->ncols);
    VK_CUDA(h, cudaMemcpy(ec.data(), h->rs.end_case, h->ncols * sizeof(int), cudaMemcpyDeviceToHost));
    for (int c = 0; c < h->ncols; ++c)
        if (ec[c] < 0) return fail(h, -ec[c], "column " + std::to_string(c) + " stopped with error " + std::to_string(-ec[c]));
    return VK_OK;
}

extern "C" int vk_run(vk_handle *h, const vk_ctrl *ctrl, int max_steps, double timeout_s) {
    return vk_run_budget(h, ctrl, max_steps, 0, timeout_s);
}

extern "C" int vk_run_budget(vk_handle *h, const vk_ctrl *ctrl, int max_steps, int max_attempts,
                             double timeout_s) {
    if (max_attempts < 0) return fail(h, VK_EINVAL, "max_attempts must be >= 0");
    vk::RunCtrl cc;
    int rc = run_prepare(h, ctrl, max_steps, cc);
    if (rc) return rc;
    cudaStream_t s = h->stream;
    const int ga = graph_attempts(cc);
    // (re)capture the attempt + control sequence when the configuration changed
    unsigned char key[sizeof(h->gkey)];
    run_key(h, cc, key);
    if (!h->gexec || std::memcmp(key, h->gkey, sizeof(key)) != 0) {
        if (h->gexec) { cudaGraphExecDestroy(h->gexec); h->gexec = nullptr; }
        cudaGraph_t g;
        VK_CUDA(h, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        run_body(h, cc, ga);
        cudaError_t ec = cudaStreamEndCapture(s, &g);
        if (ec != cudaSuccess) return fail(h, VK_ECUDA, std::string("graph capture: ") + cudaGetErrorString(ec));
        ec = cudaGraphInstantiate(&h->gexec, g, 0);
        cudaGraphDestroy(g);
        if (ec != cudaSuccess) { h->gexec = nullptr; return fail(h, VK_ECUDA, std::string("graph instantiate: ") + cudaGetErrorString(ec)); }
        std::memcpy(h->gkey, key, sizeof(key));
    }
    auto t0 = std::chrono::steady_clock::now();
    cudaEventRecord(h->ev[0], s);
    int launches = 0;
    // an attempt budget ends the call after that many attempts of the batch
    // (whole graph replays), whatever each column's step count
    const int max_replays = max_attempts > 0 ? (max_attempts + ga - 1) / ga : 0;
    for (int replay = 1;; ++replay) {
        VK_CUDA(h, cudaGraphLaunch(h->gexec, s));
        launches += body_launches(h, ga);
        int nact = 0;
        VK_CUDA(h, cudaMemcpyAsync(&nact, h->d_nactive, sizeof(int), cudaMemcpyDeviceToHost, s));
        VK_CUDA(h, cudaStreamSynchronize(s));
        if (nact == 0 || (max_replays > 0 && replay >= max_replays)) break;
        double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (timeout_s > 0 && el > timeout_s) {
            h->launches = launches;
            return fail(h, VK_ETIMEOUT, "vk_run watchdog: columns still active after " + std::to_string(el) + " s");
        }
    }
    cudaEventRecord(h->ev[1], s);
    cudaEventSynchronize(h->ev[1]);
    cudaEventElapsedTime(&h->ms[0], h->ev[0], h->ev[1]);
    h->ms[1] = h->ms[2] = h->ms[3] = 0.f;
    h->launches = launches;
    return run_check_end(h);
}

// ---------------------------------------------------------------------------
// Several handles -- one network each, any ni -- run by one graph: each
// handle's loop body on its own stream, forked from the group's stream and
// joined back, so the networks' kernels share the GPU in one launch.
struct vk_group {
    std::vector<vk_handle *> hs;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev_fork = nullptr;
    std::vector<cudaEvent_t> ev_join;   // one per handle
    cudaEvent_t ev[2] = {};
    cudaGraphExec_t gexec = nullptr;
    std::vector<unsigned char> key;
    int *h_nactive = nullptr;           // pinned [n]
    float ms = 0.f;
    int launches = 0;
};

extern "C" void vk_group_destroy(vk_group *g) {
    if (!g) return;
    if (g->stream) cudaStreamSynchronize(g->stream);
    if (g->gexec) cudaGraphExecDestroy(g->gexec);
    if (g->ev_fork) cudaEventDestroy(g->ev_fork);
    for (cudaEvent_t e : g->ev_join) if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : g->ev) if (e) cudaEventDestroy(e);
    if (g->h_nactive) cudaFreeHost(g->h_nactive);
    if (g->stream) cudaStreamDestroy(g->stream);
    delete g;
}

extern "C" int vk_group_create(vk_handle *const *handles, int n, vk_group **out) {
    if (!out) return fail(nullptr, VK_EINVAL, "out is NULL");
    *out = nullptr;
    if (!handles || n < 1) return fail(nullptr, VK_EINVAL, "a group needs at least one handle");
    for (int i = 0; i < n; ++i) {
        if (!handles[i]) return fail(nullptr, VK_EINVAL, "handle " + std::to_string(i) + " is NULL");
        for (int j = 0; j < i; ++j)
            if (handles[j] == handles[i])
                return fail(nullptr, VK_EINVAL, "handle " + std::to_string(i) + " appears twice");
    }
    vk_group *g = new (std::nothrow) vk_group();
    if (!g) return fail(nullptr, VK_ENOMEM, "out of host memory");
    g->hs.assign(handles, handles + n);
    g->ev_join.assign(n, nullptr);
    auto bad = [&](const char *what, cudaError_t e) {
        vk_group_destroy(g);
        return fail(nullptr, VK_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
    };
    cudaError_t e = cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return bad("cudaStreamCreate", e);
    if ((e = cudaEventCreateWithFlags(&g->ev_fork, cudaEventDisableTiming)) != cudaSuccess)
        return bad("cudaEventCreate", e);
    for (auto &ev : g->ev_join)
        if ((e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming)) != cudaSuccess)
            return bad("cudaEventCreate", e);
    for (auto &ev : g->ev)
        if ((e = cudaEventCreate(&ev)) != cudaSuccess) return bad("cudaEventCreate", e);
    if ((e = cudaMallocHost(&g->h_nactive, n * sizeof(int))) != cudaSuccess)
        return bad("cudaMallocHost", e);
    *out = g;
    return VK_OK;
}

extern "C" int vk_group_run(vk_group *g, const vk_ctrl *ctrls, int max_steps, int max_attempts,
                            double timeout_s) {
    if (!g) return fail(nullptr, VK_EINVAL, "group is NULL");
    if (!ctrls) return fail(nullptr, VK_EINVAL, "ctrls is NULL");
    if (max_attempts < 0) return fail(nullptr, VK_EINVAL, "max_attempts must be >= 0");
    const int n = (int)g->hs.size();
    std::vector<vk::RunCtrl> cc(n);
    for (int i = 0; i < n; ++i) {
        vk_handle *h = g->hs[i];
        int rc = run_prepare(h, &ctrls[i], max_steps, cc[i]);
        if (rc) return fail(nullptr, rc, "handle " + std::to_string(i) + ": " + h->err);
        // the group's stream starts after every handle's per-call start
        cudaEventRecord(g->ev_join[i], h->stream);
        VK_CUDA(nullptr, cudaStreamWaitEvent(g->stream, g->ev_join[i], 0));
    }
    int ga = kGraphAttempts;
    for (int i = 0; i < n; ++i) ga = std::min(ga, graph_attempts(cc[i]));
    const size_t kh = sizeof(vk_handle::gkey);
    std::vector<unsigned char> key(sizeof(int) + n * (sizeof(void *) + sizeof(unsigned) + kh));
    unsigned char *kp = key.data();
    std::memcpy(kp, &ga, sizeof(int)); kp += sizeof(int);
    for (int i = 0; i < n; ++i) {
        const vk_handle *h = g->hs[i];
        std::memcpy(kp, &h, sizeof(void *)); kp += sizeof(void *);
        std::memcpy(kp, &h->gen, sizeof(unsigned)); kp += sizeof(unsigned);
        run_key(h, cc[i], kp); kp += kh;
    }
    cudaStream_t s = g->stream;
    if (!g->gexec || key != g->key) {
        if (g->gexec) { cudaGraphExecDestroy(g->gexec); g->gexec = nullptr; }
        g->key.clear();
        cudaGraph_t graph;
        VK_CUDA(nullptr, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        cudaEventRecord(g->ev_fork, s);
        for (int i = 0; i < n; ++i) {
            vk_handle *h = g->hs[i];
            cudaStreamWaitEvent(h->stream, g->ev_fork, 0);
            run_body(h, cc[i], ga);
            cudaEventRecord(g->ev_join[i], h->stream);
            cudaStreamWaitEvent(s, g->ev_join[i], 0);
        }
        cudaError_t ec = cudaStreamEndCapture(s, &graph);
        if (ec != cudaSuccess) return fail(nullptr, VK_ECUDA, std::string("group graph capture: ") + cudaGetErrorString(ec));
        ec = cudaGraphInstantiate(&g->gexec, graph, 0);
        cudaGraphDestroy(graph);
        if (ec != cudaSuccess) { g->gexec = nullptr; return fail(nullptr, VK_ECUDA, std::string("group graph instantiate: ") + cudaGetErrorString(ec)); }
        g->key = key;
    }
    auto t0 = std::chrono::steady_clock::now();
    cudaEventRecord(g->ev[0], s);
    int launches = 0, per_replay = 0, replays = 0;
    for (int i = 0; i < n; ++i) per_replay += body_launches(g->hs[i], ga);
    const int max_replays = max_attempts > 0 ? (max_attempts + ga - 1) / ga : 0;
    for (int replay = 1;; ++replay) {
        VK_CUDA(nullptr, cudaGraphLaunch(g->gexec, s));
        launches += per_replay;
        replays = replay;
        for (int i = 0; i < n; ++i)
            VK_CUDA(nullptr, cudaMemcpyAsync(g->h_nactive + i, g->hs[i]->d_nactive, sizeof(int),
                                             cudaMemcpyDeviceToHost, s));
        VK_CUDA(nullptr, cudaStreamSynchronize(s));
        int nact = 0;
        for (int i = 0; i < n; ++i) nact += g->h_nactive[i];
        if (nact == 0 || (max_replays > 0 && replay >= max_replays)) break;
        double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (timeout_s > 0 && el > timeout_s) {
            g->launches = launches;
            return fail(nullptr, VK_ETIMEOUT, "vk_group_run watchdog: columns still active after " + std::to_string(el) + " s");
        }
    }
    cudaEventRecord(g->ev[1], s);
    cudaEventSynchronize(g->ev[1]);
    cudaEventElapsedTime(&g->ms, g->ev[0], g->ev[1]);
    g->launches = launches;
    for (int i = 0; i < n; ++i) {
        vk_handle *h = g->hs[i];
        h->ms[0] = g->ms;                 // device time of the whole group call
        h->ms[1] = h->ms[2] = h->ms[3] = 0.f;
        h->launches = replays * body_launches(h, ga);
        int rc = run_check_end(h);
        if (rc) return fail(nullptr, rc, "handle " + std::to_string(i) + ": " + h->err);
    }
    return VK_OK;
}

extern "C" int vk_group_timing(const vk_group *g, double *ms, int *launches) {
    if (!g) return fail(nullptr, VK_EINVAL, "group is NULL");
    if (ms) *ms = g->ms;
    if (launches) *launches = g->launches;
    return VK_OK;
}

extern "C" int vk_get_refine_stats(vk_handle *h, int *max_sweeps, int *n_fallback) {
    int rc = need_batch(h);
    if (rc) return rc;
    if (h->precision != VK_PREC_MIXED) {
        if (max_sweeps) *max_sweeps = 0;
        if (n_fallback) *n_fallback = 0;
        return VK_OK;
    }
    int sw = 0;
    std::vector<int> fb(h->ncols);
    VK_CUDA(h, cudaMemcpy(&sw, h->w.sweeps, sizeof(int), cudaMemcpyDeviceToHost));
    VK_CUDA(h, cudaMemcpy(fb.data(), h->w.fallback, h->ncols * sizeof(int), cudaMemcpyDeviceToHost));
    if (max_sweeps) *max_sweeps = sw;
    if (n_fallback) {
        int nf = 0;
        for (int v : fb) nf += v != 0;
        *n_fallback = nf;
    }
    return VK_OK;
}
