// Internal declarations shared by the vk_* translation units.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <vector>

#include "../../include/vk_ros2.h"

#define VK_MAXF 4              // distinct species on one side of a reaction
#define VK_CORR (1.38064852E-16 / 1.0e6)   // k_B / P0 (1 bar), the reference's gibbs corr
#define VK_MAX_NI 160          // largest species count a diagonal block may have
#define VK_MAX_NATOM 16

#define VK_MAXT 5              // written terms on one side (incl. M)

// One forward/reverse reaction pair (64 bytes).  The written-order terms
// reproduce the reference's generated rate lambdas k*t1*t2*... exactly; the
// merged factors (species with summed exponents, M separate) feed the
// Jacobian.
struct PairDesc {
    int16_t tsp[2][VK_MAXT];   // written terms per side, -1 = M, side 0 = reactants
    uint8_t tnu[2][VK_MAXT];   // coefficients of the written terms
    uint8_t nt[2];             // written-term counts
    int16_t fsp[VK_MAXF];      // merged reactant species, -1 unused
    int16_t rsp[VK_MAXF];      // merged product species
    uint8_t fnu[VK_MAXF];      // merged exponents
    uint8_t rnu[VK_MAXF];
    uint8_t nf, nr, fm, rm;    // merged counts, powers of M
    uint8_t pad[4];
};
static_assert(sizeof(PairDesc) == 64, "PairDesc layout");

// Derivative term: d v_p / d y_q (q may sit on either side).
struct WDesc {
    int pair;
    int q;
    int fpos;                  // index of q in the forward factor list or -1
    int rpos;                  // index of q in the reverse factor list or -1
};

// Host-side compiled network (what vk_network_compile builds).
struct vk_network {
    int ni = 0, npair = 0, natom = 0;
    std::vector<PairDesc> pairs;
    std::vector<int> src_ptr;          // [ni+1]
    std::vector<int2> src;             // {pair, coefficient code}  (code: +1, -1, 0 = see src_nu)
    std::vector<double> src_nu;        // coefficient of each src term
    std::vector<WDesc> w;              // derivative terms
    std::vector<int> jptr;             // [nnz+1]
    std::vector<int2> jterm;           // {w index, coefficient code}
    std::vector<double> jterm_nu;
    std::vector<int> jrow, jcol, jpos; // entry -> (s, q), s*ni+q
    std::vector<int> jrowptr;          // [ni+1] entries are sorted by row
    std::vector<int> jmap;             // [ni*ni] entry at (s, q) or -1
    std::vector<double> compo;         // [ni*natom]
    // Device form of the tables (one FP64 operation per gathered term):
    std::vector<int> porder;           // [npair] pairs by decreasing written-term count
    std::vector<int> src_slot;         // [nsrc] slot of the rate array each source term reads
    std::vector<double> src_c;         // [nsrc] signed power-of-two coefficient (exact product)
    std::vector<int> xmul_pair;        // [nxm] extra slots npair+m = xmul_fac[m] * v[xmul_pair[m]]
    std::vector<double> xmul_fac;      //       (coefficients that are not powers of two)
    std::vector<int> hk;               // [nh] rate-constant slot (2*pair + side) of half term h
    std::vector<int> hptr;             // [nh+1] factor list of h: indices into (y of the layer, M)
    std::vector<int16_t> hfac;         //        index ni stands for M
    std::vector<int> hjterm;           // [njt] half term of each Jacobian gather term
    std::vector<double> hjcoef;        // [njt] its coefficient (stoichiometry x exponent, signed)
    std::vector<int> hjptr;            // [nnz+1]
};

// Device view of the network tables (passed by value to kernels).
struct DevNet {
    int ni, npair, nr, nw, nnz, natom;
    const PairDesc *pairs;
    const int *src_ptr;
    const int *src_order;      // [ni] species by decreasing production/loss term count
    const int2 *src;
    const double *src_nu;
    const WDesc *w;
    const int *jptr;
    const int *jorder;         // [nnz] Jacobian entries by decreasing term count
    const int2 *jterm;
    const double *jterm_nu;
    const int *jpos;
    const int *jrow, *jcol, *jrowptr, *jmap;
    const double *compo;
    // the gather form (vk_network): pair order, source slots and coefficients,
    // extra products, derivative half terms, Jacobian gather terms
    int nxm, nh;
    const int *porder;
    const int *src_slot;
    const double *src_c;
    const int *xmul_pair;
    const double *xmul_fac;
    const int *hk, *hptr;
    const int16_t *hfac;
    const int *hjterm, *hjptr;
    const double *hjcoef;
};

// Device view of a loaded batch of columns.
struct DevBatch {
    int ncols;
    int L;                     // total layers
    const int *col_off;        // [ncols+1] first layer of each column
    const int *col_end;        // [ncols] one past its last layer (col_off[c+1] when packed;
                               //  slots of a fixed capacity leave gap layers between)
    const int *lay_col;        // [L] column of each layer, -1 for a gap layer
    const double *k;           // [L][nr]
    const double *atm;         // [L][VK_ATM_NF]
    const double *Dzz;         // [L][ni]
    const double *spf;         // [ncols][VK_SP_NF][ni]
    const int *active;         // [ncols] non-zero = column takes part (NULL = all)
    const int *order;          // [ncols] columns by decreasing nz (work-queue order)
    unsigned *queue;           // [1] next queue position (zeroed before each launch)
    int nsm;                   // SMs of the device
    int cps;                   // resident CTAs per SM of the per-column kernels
                               // (0: each kernel's own default)
    int cps_k[VK_TUNE_N];      // per-kernel setting of vk_set_launch (0: cps)
    int lu32_tiling;           // k_lu32 register tiling (-1: by ni)
    int grid_rates, grid_prep; // CTAs of the per-layer kernels k_rates / k_prep32:
                               // all of them resident at once, each striding over
                               // the layers (0: one CTA per layer)
};

// Grid of a per-layer kernel whose CTAs stride over the layers: as many CTAs
// as fit on the device at once (per_sm of them per SM), at most one per layer.
inline int layer_grid(const DevBatch &b, int want) {
    return want > 0 && want < b.L ? want : (b.L > 0 ? b.L : 1);
}

// Doubles per FP64 block of the n x n inverses in global memory: n*n rounded
// up to even, so every block starts on 16 bytes (bulk-copy alignment).
__host__ __device__ inline int block_stride64(int n) { return (n * n + 1) & ~1; }

// Raise a kernel's dynamic shared-memory limit to at least `bytes`, never
// lowering it: handles of different networks share the kernels, and a loop
// captured for the larger network must stay launchable after a smaller
// network's handle is created.
template <typename K>
inline cudaError_t raise_smem_limit(K *kernel, size_t bytes) {
    cudaFuncAttributes a;
    cudaError_t e = cudaFuncGetAttributes(&a, kernel);
    if (e != cudaSuccess) return e;
    if ((size_t)a.maxDynamicSharedSizeBytes >= bytes) return cudaSuccess;
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

// Grid of a per-column kernel: CTAs per SM from vk_set_launch, else the
// batch's override, else the kernel's default; never more than the columns.
inline int column_grid(const DevBatch &b, int kernel, int cps_default) {
    const int cps = b.cps_k[kernel] > 0 ? b.cps_k[kernel] : b.cps > 0 ? b.cps : cps_default;
    const long long g = (long long)cps * b.nsm;
    return (g > 0 && g < b.ncols) ? (int)g : b.ncols;
}

#ifdef __CUDACC__
// Per-column kernels run as a work queue: each CTA takes the next column in
// b.order (longest first) until the queue is empty, so the SMs finish
// together however uneven the columns are.  All threads call it; returns -1
// when no column is left.
__device__ __forceinline__ int next_column(const DevBatch &b, int *s_col) {
    __syncthreads();                 // everyone has read the previous s_col
    if (threadIdx.x == 0) {
        const unsigned i = atomicAdd(b.queue, 1u);
        *s_col = i < (unsigned)b.ncols ? b.order[i] : -1;
    }
    __syncthreads();
    return *s_col;
}
#endif

// Photochemistry radiative transfer tables and state (vk_photo.cu).
struct PhotoDev {
    int nbins, nabs, nscat, nch;
    const double *bins;        // [nbins] wavelength (nm)
    const double *cross;       // [nabs][nbins] absorption cross sections
    const int *abs_sp;         // [nabs] species index
    const int *abs_photo;      // [nabs] 1: counts in the absorption of the albedo
    const double *cross_scat;  // [nscat][nbins] Rayleigh cross sections
    const int *scat_sp;        // [nscat]
    const double *wcross_J;    // [nch][nbins] photolysis cross section x J bin weight
    const int *ch_kindex;      // [nch] 1-based k index of the channel
    const double *sflux_top;   // [nbins] top-of-atmosphere flux
    double sl_angle, edd, f_diurnal, flux_atol;
    double *tau, *dflux_u, *dflux_d;   // [(L + ncols)][nbins] staggered
    double *w0, *aflux, *aflux_prev;   // [L][nbins]
    double *J;                 // [L][nch]
    // temperature-dependent cross sections (vk_photo_set_cross_T); NULL: none
    const int *abs_tslot;      // [nabs] row of cross_T, or -1
    const double *cross_T;     // [nabs_t][lstride][nbins]
    const int *ch_tslot;       // [nch] row of wcross_J_T, or -1
    const double *wcross_J_T;  // [nch_t][lstride][nbins] x J bin weight
    int lstride;               // layer stride of the per-layer tables
};

// Launch helpers implemented in vk_kernels.cu (all asynchronous on stream).
namespace vk {

constexpr double R_ROS = 1.0 + 0.70710678118654752440;   // 1 + 1/sqrt(2)

// Message returned by vk_last_error(NULL) on this thread (not exported).
void set_global_error(const std::string &msg);

struct Work {                  // per-handle device work buffers
    double *y, *ymix, *yk2, *f, *k1, *k2, *z, *sol, *ymix_out;
    double *jv;                // [L][nnz]  -J_chem entries
    double *dA, *dB, *dC;      // [L][ni]   diffusion coefficients (A+Ai, B+Bi, C+Ci)
    double *geo;               // [L][5][ni] state-free transport geometry (vk_geo.cuh)
    double *G;                 // [L][block_stride64(ni)] FP64 block inverses
    float *G32;                // [L][ni*ni] FP32 inverses of the scaled blocks (mixed mode)
    double *rs, *cs;           // [L][ni] power-of-two row / column scales (mixed mode)
    double *r;                 // refinement residual
    double *f2;                // [L][ni] second-stage right-hand side (mixed mode)
    float *zf;                 // [L][ni] FP32 forward-sweep vector (mixed mode)
    float *wcf, *wcb;          // [L][ni] scaled couplings of the refinement sweeps (mixed mode)
    float *raf;                // [L][ni] scaled residual of the current sweep (mixed mode)
    float *xf;                 // [L][ni] back-sweep result of the current sweep (mixed mode)
    float *D32;                // [L][stride] dense scaled FP32 blocks (mixed mode)
    int *fallback;             // [ncols] attempt solved in FP64 (routed or refinement failed)
    int *act32;                // [ncols] attempt solved by the FP32 factors + refinement
    int *routed;               // [ncols] attempt solved in FP64 from the start (routing)
    int *failed;               // [ncols] refinement failed: redone in FP64 after the others
    double *thr64;             // [ncols] step size at which refinement last failed: an
                               //         attempt with dt >= thr64 goes straight to FP64
    int *sweeps;               // [1] most refinement sweeps any column needed
    double *refine_err;        // [ncols] last accepted correction size of the attempt
    double *dt;                // [ncols]
    double *delta;             // [ncols]
    int *status;               // [ncols]  VK_* per column (singular pivot ...)
    const void *tmap_d32;      // host: CUtensorMap over D32 as k_lu_tc's padded tiles
};

void launch_rates(const DevNet &net, const DevBatch &b, const double *y, double *f,
                  double *jv, double *dA, double *dB, double *dC, const double *k1,
                  const double *dt, const double *geo, int flags, bool with_jac, cudaStream_t s);
void launch_geometry(const DevNet &net, const DevBatch &b, double *geo, int flags, cudaStream_t s);
void launch_lu_fwd_f64(const DevNet &net, const DevBatch &b, const Work &w,
                       const double *rhs, double *z, int flags, cudaStream_t s);
void launch_back_f64(const DevNet &net, const DevBatch &b, const double *G,
                     const double *dB, const double *z, double *x,
                     const double *y, double *yk2, int *status, cudaStream_t s);
void launch_solve_f64(const DevNet &net, const DevBatch &b, const double *G,
                      const double *dB, const double *dC, const double *rhs,
                      double *zbuf, double *x, int *status, cudaStream_t s);
void launch_stage(const DevNet &net, const DevBatch &b, const Work &w, int flags,
                  double mtol, double atol, cudaStream_t s);
void launch_refine(const DevNet &net, const DevBatch &b, const Work &w, const double *rhs,
                   double *x, const double *yscale, double *yk2, int max_sweeps, double tol,
                   cudaStream_t s);
void launch_rate_consts(const DevNet &net, const DevBatch &b, const int *kind, const int *rev,
                        const int *cap_kind, const double *cap_T, const double *cap_params,
                        const double *params, const double *nasa9, double *k, cudaStream_t s);
void launch_photo(const DevNet &net, const DevBatch &b, const PhotoDev &ph, const double *y,
                  const double *ymix, double *k, unsigned long long *change, cudaStream_t s);
void launch_photo_clear(const DevBatch &b, unsigned long long *change, cudaStream_t s);
void launch_route(const DevBatch &b, const Work &w, cudaStream_t s);
void launch_reset_route(const Work &w, int ncols, double route_dt0, cudaStream_t s);
cudaError_t init_mixed_kernels(int n);
cudaError_t init_lureg_kernels(const DevNet &net);
// Resident CTAs per SM of the per-layer kernels for a network (0: unknown);
// call after the init_* functions have raised their shared-memory limits.
int rates_blocks_per_sm(const DevNet &net);
int prep_blocks_per_sm(const DevNet &net);
void launch_lu_reg32(const DevNet &net, const DevBatch &b, const Work &w, cudaStream_t s);
int lu32_tiling_cap(int tiling);     // largest block a k_lu32 tiling covers (0: none)
// tensor-core factorisation (vk_lutc.cu): the LU32 tiling values that select
// it with the one-warp panel and with the four-warp cooperative panel
constexpr int VK_LU_TC = 4;
constexpr int VK_LU_TC_COOP = 5;
bool lu_tc_supported(int n);
cudaError_t lu_tc_make_map(CUtensorMap *map, const float *D32, int n, int max_layers);
void launch_lu_tc(const DevNet &net, const DevBatch &b, const Work &w, const CUtensorMap &map,
                  bool coop, cudaStream_t s);
size_t lu_tc_block_floats(int n);    // floats per layer of its padded scaled blocks
cudaError_t init_lu_tc(int n);

}  // namespace vk
