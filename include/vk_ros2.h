/*
 * vk_ros2.h -- C ABI of the GB300-native VULCAN Ros2 kinetics-diffusion step.
 *
 * Plain C types only (ints, doubles, pointers and sizes); host arrays are
 * caller-owned and copied in/out; device buffers are owned by the handle.
 * No C++ exception crosses this boundary: every entry point returns a
 * status code (VK_OK = 0) and vk_last_error() gives the message.
 *
 * Reference interfaces replaced (paths inside the VULCAN project):
 *   vk_network_compile  make_chem_funs.py:17-430 (network -> chemdf/df tables)
 *                       and make_chem_funs.py:653-717 (symbolic Jacobian)
 *   vk_set_columns      store.py:21-180 data contract (var.y, var.k, atm.*)
 *   vk_ros2_attempt     op.py:2860-3007   Ros2.solver (one Rosenbrock attempt)
 *   vk_run              op.py:808-936     Integration.__call__ for a batch of
 *                       columns: Ros2.one_step op.py:3091-3103 with clip /
 *                       loss / step_ok / step_reject op.py:2447-2534,
 *                       step_size op.py:3105-3125, update_mu_dz op.py:944-984,
 *                       conv / stop op.py:1018-1085 (max_steps = 1: one step)
 *   vk_get_state        var.y / var.ymix / var.dt / para.delta read-back
 *   vk_compute_k        op.py:63-342      ReadRate read_rate / rev_rate /
 *                       lim_lowT_rates on the device
 *   vk_photo_*          op.py:2580-2786   compute_tau / compute_flux /
 *                       compute_J on the device
 */
#ifndef VK_ROS2_H
#define VK_ROS2_H

#if defined(__GNUC__)
#define VK_API __attribute__((visibility("default")))
#else
#define VK_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define VK_OK            0
#define VK_EINVAL        1   /* bad argument / size beyond the handle's limits */
#define VK_ECUDA         2   /* CUDA runtime error */
#define VK_ESINGULAR     3   /* zero pivot in a diagonal block */
#define VK_ENAN          4   /* non-finite value in the state */
#define VK_EMAXATTEMPT   5   /* attempt cap reached without an accepted step */
#define VK_ETIMEOUT      6   /* host watchdog gave up waiting */
#define VK_ENOMEM        7   /* device allocation failed */

/* ---- linear-solve precision ---- */
#define VK_PREC_FP64     0   /* FP64 block LU (matches the reference step) */
#define VK_PREC_MIXED    1   /* FP32 scaled block LU + FP64 iterative refinement */

/* ---- per-layer atmosphere fields (vk_set_columns, atm[L][VK_ATM_NF]) ----
 * Interface quantities of layer j describe interface j+1/2 and are unused on
 * the top layer of a column. */
#define VK_ATM_M      0   /* third-body density M = n_0 at set-up (cm^-3)     */
#define VK_ATM_N0     1   /* total density n_0 (hydrostatic renormalisation)  */
#define VK_ATM_TCO    2   /* temperature (K)                                  */
#define VK_ATM_G      3   /* gravity g(z)                                     */
#define VK_ATM_DZI    4   /* dzi, interface spacing                           */
#define VK_ATM_KZZ    5   /* eddy diffusion at the interface                  */
#define VK_ATM_VZ     6   /* vertical wind at the interface                   */
#define VK_ATM_TI     7   /* interface temperature Ti                         */
#define VK_ATM_HPI    8   /* interface scale height Hpi                       */
#define VK_ATM_HP     9   /* layer scale height Hp (steady-state slope)       */
#define VK_ATM_PICO  10   /* pressure at the lower interface of the layer     */
#define VK_ATM_PICOU 11   /* pressure at the upper interface of the layer     */
#define VK_ATM_DZ    12   /* layer thickness dz                               */
#define VK_ATM_NF    13

/* ---- per-column species fields (vk_set_columns, spf[col][VK_SP_NF][ni]) ---- */
#define VK_SP_MS        0   /* molar mass                                     */
#define VK_SP_ALPHA     1   /* thermal diffusion factor                       */
#define VK_SP_TOPFLUX   2
#define VK_SP_BOTFLUX   3
#define VK_SP_BOTVDEP   4
#define VK_SP_NF        5

/* ---- flags ---- */
#define VK_F_MOLDIFF    1   /* vulcan_cfg.use_moldiff: diffdf / lhs_jac_tot   */
#define VK_F_TOPFLUX    2   /* vulcan_cfg.use_topflux                          */
#define VK_F_BOTFLUX    4   /* vulcan_cfg.use_botflux                          */

/* Network description, in the written order of the network file.  Reaction
 * pair p has forward k index 2p+1 and reverse 2p+2 (rows 2p and 2p+1 of the
 * rate array).  Each side lists its terms as written ("H + H + M" is three
 * terms, "2*X" one term with coefficient 2); species index -1 denotes M. */
typedef struct vk_network_desc {
    int ni;                 /* number of species                              */
    int npair;              /* number of forward/reverse reaction pairs       */
    const int *reac_ptr;    /* [npair+1] CSR into reac_sp / reac_nu           */
    const int *reac_sp;     /* species index, -1 = M                          */
    const int *reac_nu;     /* stoichiometric coefficient                     */
    const int *prod_ptr;    /* [npair+1] CSR into prod_sp / prod_nu           */
    const int *prod_sp;
    const int *prod_nu;
    int natom;              /* elements tracked by the conservation check     */
    const double *compo;    /* [ni * natom] element counts                    */
} vk_network_desc;

typedef struct vk_network vk_network;   /* compiled tables (host memory)     */
typedef struct vk_handle vk_handle;     /* device state for a batch          */

/* Solver controls (defaults = the reference's vulcan_cfg values). */
typedef struct vk_ctrl {
    double rtol, atol, mtol, mtol_conv, pos_cut, nega_cut, loss_eps;
    double dt_min, dt_max, dt_var_min, dt_var_max;
    double yconv_cri, slope_cri, yconv_min, st_factor, trun_min, runtime;
    int conv_step, count_min, count_max, update_frq;
    int max_attempts;       /* attempt cap per step (device guard)            */
    int flags;              /* VK_F_* */
    double gs, Rp;          /* gravity update (update_mu_dz)                  */
    double flux_cri;        /* steady state also needs the actinic-flux change
                               of the last vk_photo_update below this
                               (op.py:1054; 0 change without photochemistry) */
} vk_ctrl;

/* ---- network ---- */
VK_API int  vk_network_compile(const vk_network_desc *desc, vk_network **out);
/* sizes of the compiled tables: Jacobian non-zeros per diagonal block,
 * derivative terms, production/loss terms */
VK_API int  vk_network_info(const vk_network *net, int *nnz_jac, int *n_dterm, int *n_src);
/* Jacobian sparsity: row and column of each stored entry (arrays of nnz_jac) */
VK_API int  vk_network_jac_pattern(const vk_network *net, int *rows, int *cols);
/* Diagnostic: one layer's chemical source (the generated chemdf) and its -J
 * entries (neg_symjac, in vk_network_jac_pattern order) evaluated on the host
 * from the compiled gather tables with the rate kernel's own operations and
 * order -- for checking the tables without a GPU.  y [ni], k [2*npair]
 * (forward/reverse per pair), M the layer's total number density; either
 * output may be NULL.  The reference's counterparts: chem_funs.chemdf and
 * neg_symjac generated by make_chem_funs.py:113-430, 686-717. */
VK_API int  vk_network_eval_host(const vk_network *net, const double *y, const double *k, double M,
                                 double *dydt, double *neg_jac);
VK_API void vk_network_free(vk_network *net);

/* ---- handle ---- */
VK_API int  vk_create(const vk_network *net, int max_cols, int max_layers, int precision,
               vk_handle **out);
VK_API void vk_destroy(vk_handle *h);
VK_API const char *vk_last_error(const vk_handle *h);   /* h may be NULL */
/* Switch the linear-solve precision; max_refine caps the refinement sweeps
 * (default 6) and refine_tol is the convergence test on the correction
 * relative to |x| + |y| + 1e-10 n_0 (default 1e-10). */
VK_API int  vk_set_precision(vk_handle *h, int precision, int max_refine, double refine_tol);
/* Mixed precision: the step size from which a column's attempts go straight
 * to the FP64 solve (default INFINITY: every column tries the FP32 factors
 * until its refinement first fails, then uses FP64 from a quarter of that
 * step on).  A finite dt0 spares a column its first failure when the
 * caller knows where FP32 factors stop preconditioning these systems (a
 * failed refinement is redone in FP64 after the attempt's other solves, a
 * serial FP64 chain).  Applies to every column now and at its next start;
 * a failure still lowers a column's limit.  No counterpart in the reference,
 * which solves every step in FP64 (op.py:2913-2929). */
VK_API int  vk_set_route(vk_handle *h, double dt0);

/* Load a batch of columns.  L = sum(nz).  k is [L][2*npair] (layer-major,
 * row l holds k[1..nr] of that layer), atm is [L][VK_ATM_NF], Dzz is [L][ni]
 * (interface values, top layer unused), spf is [ncols][VK_SP_NF][ni],
 * y and ymix are [L][ni].  Copies everything to the device. */
VK_API int  vk_set_columns(vk_handle *h, int ncols, const int *nz, const double *k,
                    const double *atm, const double *Dzz, const double *spf,
                    const double *y, const double *ymix);
/* The same set-up in the slotted layout used for continuous batching (no
 * counterpart in the reference, which integrates one column per run): column
 * c occupies layers c*slot_cap .. c*slot_cap + nz[c] - 1 of the device arrays
 * ([ncols*slot_cap] layers; the rest of each slot holds no column), so a
 * finished column can be replaced by vk_refill without moving the others.
 * Inputs are packed as for vk_set_columns; requires nz[c] <= slot_cap and
 * ncols*slot_cap <= max_layers.  Outputs indexed by layer (vk_get_state,
 * vk_ros2_attempt, ...) use the slotted layout. */
VK_API int  vk_set_columns_slotted(vk_handle *h, int ncols, int slot_cap, const int *nz,
                                   const double *k, const double *atm, const double *Dzz,
                                   const double *spf, const double *y, const double *ymix);
/* Continuous batching: put n new columns into the given slots (slotted
 * layout only), packed inputs as vk_set_columns, plus their element totals
 * atom_ini [n][natom] (vk_set_atom_ini), 1-bar reference levels pref_indx
 * [n] and steady-state ignore masks conv_ignore [n][ni] (NULL: keep the
 * slot's).  Each refilled column starts a run: t = 0, count = 0, dt = 1e-10,
 * end_case 0, its history and routing reset; the other columns are
 * untouched.  The loop it feeds is Integration.__call__ (op.py:808-936), run
 * per column. */
VK_API int  vk_refill(vk_handle *h, int n, const int *slots, const int *nz, const double *k,
                      const double *atm, const double *Dzz, const double *spf,
                      const double *y, const double *ymix, const double *atom_ini,
                      const int *pref_indx, const int *conv_ignore);
/* Update only the fields that change during a run (y, ymix, atm, k). */
VK_API int  vk_update_state(vk_handle *h, const double *y, const double *ymix);
VK_API int  vk_update_atm(vk_handle *h, const double *atm);
VK_API int  vk_update_k(vk_handle *h, const double *k);

/* One Ros2 attempt for every column with its own dt[col] (op.py:2860-3007):
 * outputs sol (written to the device y), ymix, delta[col]; k1/k2 optional
 * (NULL to skip the copy-out).  flags = VK_F_*. */
VK_API int  vk_ros2_attempt(vk_handle *h, const double *dt, int flags, double *sol,
                     double *ymix, double *delta, double *k1, double *k2);

/* Element totals at set-up (InitialAbun.ele_sum) used by the loss check. */
VK_API int  vk_set_atom_ini(vk_handle *h, const double *atom_ini /*[ncols][natom]*/);

/* Per-column index of the 1-bar reference interface (f_mu_dz pref_indx) and
 * a per-species mask [ni] of species ignored by the steady-state test
 * (vulcan_cfg.conver_ignore); either pointer may be NULL. */
VK_API int  vk_set_column_info(vk_handle *h, const int *pref_indx, const int *conv_ignore);
/* Per-column masks [ncols][ni] of species the steady-state test ignores (the
 * conver_ignore list of each column's cfg, op.py:1043-1045); replaces the one
 * mask vk_set_column_info gives every column. */
VK_API int  vk_set_conv_ignore(vk_handle *h, const int *conv_ignore);

/* Integrate every column on the device until each one reaches steady state
 * or a limit (count_max / runtime), or until max_steps accepted steps per
 * column have been taken in this call (0 = no cap).  dt/t/count live on the
 * device; the loop is captured once into a CUDA graph of 8 attempts (of
 * max_steps attempts when max_steps < 8) and replayed. */
VK_API int  vk_run(vk_handle *h, const vk_ctrl *ctrl, int max_steps, double timeout_s);
/* vk_run with an attempt budget as well: the call also returns once the
 * batch has made max_attempts attempts (rounded up to the graph's length; 0 = no
 * budget), the columns keeping their state for the next call.  For
 * continuous batching: a column whose steps need many rejected attempts
 * then holds the batch for at most the budget, while the others' slots are
 * refilled between calls.  Same loop as op.py:808-936 per column. */
VK_API int  vk_run_budget(vk_handle *h, const vk_ctrl *ctrl, int max_steps, int max_attempts,
                          double timeout_s);

/* Several networks in one launch.  A group holds handles of any networks
 * (any ni, each with its own columns, precision and launch settings); one
 * vk_group_run runs all of them to steady state like vk_run_budget does each,
 * with every handle's loop body (attempts + control) on its own stream inside
 * one CUDA graph, forked from the group's stream and joined back, so the
 * networks' kernels share the GPU in one graph launch per replay.  Each
 * handle's results are bit for bit those of vk_run_budget on that handle
 * alone: the kernels and their inputs are the same; only their placement in
 * time differs.  Destroy the group before its handles.  Errors of these
 * calls are read with vk_last_error(NULL); an error of one handle's run is
 * reported as "handle i: <its message>".  The per-column loop they replace
 * is op.py:808-936, run once per column. */
typedef struct vk_group vk_group;
VK_API int  vk_group_create(vk_handle *const *handles, int n, vk_group **out);
/* ctrls: n control structs, one per handle in group order; max_steps,
 * max_attempts and timeout_s as in vk_run_budget, for the whole group. */
VK_API int  vk_group_run(vk_group *g, const vk_ctrl *ctrls, int max_steps, int max_attempts,
                         double timeout_s);
/* Device time of the last vk_group_run (ms) and the kernels it launched. */
VK_API int  vk_group_timing(const vk_group *g, double *ms, int *launches);
VK_API void vk_group_destroy(vk_group *g);

/* Per-column state read-back: y/ymix [L][ni]; the scalar arrays are [ncols]
 * (NULL to skip).  end_case: 0 running, 1 converged, 2 runtime, 3 count_max,
 * negative = error status. */
VK_API int  vk_get_state(vk_handle *h, double *y, double *ymix, double *dt, double *t,
                  int *count, int *end_case, double *delta);
/* Initial dt / t / count per column before vk_run (dt = vulcan_cfg.dttry). */
VK_API int  vk_set_clock(vk_handle *h, const double *dt, const double *t, const int *count);

/* Cumulative counters per column: [ncols][VK_NCOUNTERS] = attempts, delta
 * rejections, negativity rejections, loss rejections, attempts solved in FP64
 * on a mixed-precision handle (routed there because refinement had failed at
 * that step size, or redone after it failed), accepted steps. */
#define VK_NCOUNTERS 6
VK_API int  vk_get_counters(vk_handle *h, int *counters);
/* Diagnostic: longdy and longdydt of each column's last steady-state test
 * (the reference keeps them as var.longdy / var.longdydt, op.py:1046-1049). */
VK_API int  vk_get_conv(vk_handle *h, double *longdy, double *longdydt);

/* Device time of the last call in ms: after vk_ros2_attempt the rate +
 * Jacobian kernel, the block factorisation, the solves (including the second
 * right-hand side and any FP64 fallback) and the stage kernel; after vk_run
 * ms_rates holds the whole run and the others are 0.  launches = kernels
 * launched by the call. */
VK_API int  vk_get_timing(vk_handle *h, double *ms_rates, double *ms_lu, double *ms_solve,
                   double *ms_stage, int *launches);

/* ---- rate constants on the device ----
 * Replaces the host's op.ReadRate.read_rate / rev_rate (op.py:63-309) for
 * batches whose temperature varies by column.  Per reaction pair: kind
 * (VK_K_*), rev = 1 when the reverse rate is k_f / Keq (pairs before
 * '# reverse stops'), params = A B C A_inf B_inf C_inf; nasa9 [ni][20] with
 * the T < 1000 K range first (chem_funs gibbs_sp).  vk_compute_k fills the
 * device k of every layer from the atmosphere's TCO and M; forward slots of
 * VK_K_NONE pairs (photolysis, ionisation, condensation) keep the uploaded
 * values (frozen J). */
#define VK_K_NONE           0
#define VK_K_ARRHENIUS      1
#define VK_K_FALLOFF        2
#define VK_K_SPECIAL_OH_CH3 3
VK_API int  vk_set_rate_params(vk_handle *h, const int *kind, const int *rev, const double *params,
                               const double *nasa9);
/* Low-temperature caps (use_lowT_limit_rates; op.ReadRate.lim_lowT_rates,
 * op.py:320-342): per pair, kind VK_K_NONE (no cap), VK_K_ARRHENIUS or
 * VK_K_FALLOFF with params [6] as in vk_set_rate_params; where the layer's
 * T <= t_max, vk_compute_k takes the cap's form as the forward rate and
 * forms the reverse rate from it (the reference's order).  kind = NULL
 * removes the caps. */
VK_API int  vk_set_rate_caps(vk_handle *h, const int *kind, const double *t_max,
                             const double *params);
VK_API int  vk_compute_k(vk_handle *h);
/* ---- launch tuning (for an autotuner; no counterpart in the reference) ----
 * The per-column kernels take columns from a work queue; their grid is
 * ctas_per_sm x SMs CTAs.  kernel: VK_TUNE_*; ctas_per_sm 0..8 (0: the
 * kernel's built-in default, or VK_CTAS_PER_SM from the environment);
 * variant: for VK_TUNE_LU32 the register tiling of the FP32 Gauss-Jordan,
 * 0..3 covering blocks up to 48, 80, 112, 160 species, 4: the tensor-core
 * factorisation (tcgen05, blocks up to 128 species) with one warp eliminating
 * each 16-pivot panel, or 5: the same with the four warps of its CTA
 * eliminating the panel together (identical factors) (-1: the default for
 * ni, variant 5 up to 128 species; a variant smaller than ni is refused),
 * ignored otherwise.
 * A change drops the captured vk_run graph, which is captured again. */
#define VK_TUNE_LU32    0   /* k_lu32: FP32 block-Thomas factorisation        */
#define VK_TUNE_LU64    1   /* k_lu_fwd_f64: FP64 factorisation + first sweep */
#define VK_TUNE_SWEEP64 2   /* k_back_f64, k_solve_f64: FP64 sweeps           */
#define VK_TUNE_REFINE  3   /* k_refine: FP64 refinement with FP32 factors    */
#define VK_TUNE_N       4
VK_API int  vk_set_launch(vk_handle *h, int kernel, int ctas_per_sm, int variant);
VK_API int  vk_get_launch(vk_handle *h, int kernel, int *ctas_per_sm, int *variant);
/* Diagnostic: the device rate constants [L][nr] back to the host. */
VK_API int  vk_get_k(vk_handle *h, double *k);

/* ---- photochemistry radiative transfer ----
 * op.ODESolver.compute_tau / compute_flux / compute_J (op.py:2580-2786;
 * isotropic scattering; T-dependent cross sections through
 * vk_photo_set_cross_T below) for every column.  The
 * tables are those of the reference's make_bins_read_cross / read_sflux
 * (op.py:495-782, build_atm.py:617-656): wavelength bins, the J integral's
 * bin weights, absorbers (species index, 1 if a photolysis species -- the
 * albedo's absorption counts those), their cross sections [nabs][nbins],
 * Rayleigh scatterers and cross sections [nscat][nbins], photolysis channels
 * (1-based k index of the channel's rate) and cross sections [nch][nbins],
 * the top-of-atmosphere flux [nbins]; angles in radians.  The diffuse fluxes
 * persist between updates as the reference's arrays do (vk_photo_reset
 * clears them).  vk_photo_update computes tau, the actinic flux and J from
 * the current state of the columns with col_mask[c] != 0 (NULL: all), writes
 * J * f_diurnal into the channels' k slots and each column's largest
 * relative actinic-flux change where the flux exceeds flux_atol
 * (var.aflux_change) into the run state -- the steady-state test of vk_run
 * requires it below vk_ctrl.flux_cri -- and into aflux_change if given.  No
 * counterpart for photoionisation yet. */
VK_API int  vk_photo_setup(vk_handle *h, int nbins, const double *bins, const double *jweights,
                           int nabs, const int *abs_sp, const int *abs_photo, const double *cross,
                           int nscat, const int *scat_sp, const double *cross_scat, int nch,
                           const int *ch_kindex, const double *cross_J, const double *sflux_top,
                           double sl_angle, double edd, double f_diurnal, double flux_atol);
/* Temperature-dependent cross sections (vulcan_cfg.T_cross_sp): per-layer
 * tables replacing, in the optical depth, the absorption cross section of
 * some absorbers and, in J, the photolysis cross section of some channels --
 * var.cross_T / var.cross_J_T of op.ReadRate.make_bins_read_cross
 * (op.py:640-745) as compute_tau (op.py:2591-2592) and compute_J
 * (op.py:2770-2774) read them; the single-scattering albedo keeps the
 * T-independent cross sections (op.py:2623-2624).  abs_slot[i] / ch_slot[i]:
 * position in vk_photo_setup's absorber / channel list (each at most once);
 * cross_T [nabs_t][L][nbins] and cross_J_T [nch_t][L][nbins] over the layers
 * of the current batch (call after vk_set_columns, again when the columns
 * change).  Replaces earlier tables; nabs_t = nch_t = 0 removes them. */
VK_API int  vk_photo_set_cross_T(vk_handle *h, int nabs_t, const int *abs_slot,
                                 const double *cross_T, int nch_t, const int *ch_slot,
                                 const double *cross_J_T);
VK_API int  vk_photo_reset(vk_handle *h);
VK_API int  vk_photo_update(vk_handle *h, const int *col_mask, double *aflux_change);
/* Diagnostic: tau [(L + ncols)][nbins] (staggered, column c from row
 * col_off[c] + c), actinic flux [L][nbins], J [L][nch]. */
VK_API int  vk_photo_get(vk_handle *h, double *tau, double *aflux, double *J);

/* ---- learned warm start: BF16 MLP kernels ----
 * No counterpart in the reference (its initial state comes from ini_mix,
 * build_atm.py:141-279).  Device pointers owned by the caller; BF16 weights
 * and activations, FP32 accumulation, FP32 biases/gradients/optimiser state.
 * X [B][K] bf16, W [K][N] bf16 (row-major), Z [B][N] f32, H [B][N] bf16. */
/* Z = X W + bias; H = silu(Z) (silu_act = 1) or Z.  Z or H may be NULL. */
VK_API int  vk_mlp_forward(int B, int K, int N, const void *X, const void *W, const float *bias,
                           float *Z, void *H, int silu_act, void *stream);
/* dZ = dH o silu'(Z) into dZ_scratch [B][N] bf16; dW = X^T dZ [K][N];
 * db = column sums of dZ [N]; dX = dZ W^T [B][K] (each output may be NULL). */
VK_API int  vk_mlp_backward(int B, int K, int N, const void *X, const void *W, const float *Z,
                            const float *dH, int silu_act, void *dZ_scratch, float *dW,
                            float *db, float *dX, void *stream);
/* One Adam step on n parameters (w FP32 master, optional BF16 copy). */
VK_API int  vk_mlp_adam(long long n, float *w, void *w_bf16, const float *g, float *m, float *v,
                        float lr, float beta1, float beta2, float eps, int step, void *stream);

/* ---- block-tridiagonal solve without allocation ----
 * No counterpart in the reference.  For callers that cannot call cudaMalloc
 * (a framework that owns all device memory through its own pool, a plugin
 * that is handed its buffers): the solver's scratch (block inverses and sweep vector) is a fixed 16 MiB
 * __device__ array inside this library, held by every GPU that loads it until
 * the process exits.  Solves lower[j] o x[j-1] + D[j] x[j] + upper[j] o x[j+1]
 * = b[j] for one column; D is [nz][ni][ni], lower/upper/b/x are [nz][ni], all
 * device pointers supplied by the caller; lower[0] and upper[nz-1] are not
 * read.  Requires nz*ni*ni + nz*ni + 1 <= 2^21 (e.g. nz = 200 at ni = 100);
 * larger sizes return VK_EINVAL.  Runs on `stream` (a cudaStream_t, NULL for
 * the default stream) and synchronizes it to return VK_ESINGULAR / VK_ENAN,
 * so it cannot be called while any stream is being captured into a graph.
 * The first call on a device resolves the array's address on that device.
 * All calls share the one array: calls
 * that overlap on the GPU (other threads or streams) race; serialize them.
 * Errors: vk_last_error(NULL). */
VK_API int  vk_block_solve_noalloc(int nz, int ni, const double *D, const double *lower,
                                   const double *upper, const double *b, double *x,
                                   void *stream);

/* ---- diagnostics (used by the parity tests) ---- */
/* Mixed precision, last attempt: the most refinement sweeps any column
 * needed, and how many columns were redone in FP64 (0/0 in FP64 mode). */
VK_API int  vk_get_refine_stats(vk_handle *h, int *max_sweeps, int *n_fallback);
/* Message of the last failed vk_network_compile on this thread. */
VK_API const char *vk_network_last_error(void);
/* Chemistry source term alone (the generated chemdf) of state y [L][ni]. */
VK_API int  vk_chem_source(vk_handle *h, const double *y, double *dydt);
/* Right-hand side f(y) = chemdf + diffdf of state y [L][ni] (the handle's
 * state when y is NULL) with the transport terms `flags` selects (VK_F_*):
 * the f of Ros2.solver (op.py:2888); f is [L][ni].  Leaves the handle's
 * state and its last attempt untouched. */
VK_API int  vk_rhs(vk_handle *h, const double *y, int flags, double *f);
/* FP32 inverses of the scaled diagonal blocks of the last mixed-precision
 * attempt, [L][ni*ni] row-major (columns that attempt solved in FP64 hold
 * stale values). */
VK_API int  vk_get_lu32(vk_handle *h, float *G);
/* LHS pieces of the last attempt: -J entries [L][nnz_jac] in the order of
 * vk_network_jac_pattern, and the transport coefficients dA/dB/dC [L][ni]
 * (dy_j/dt = dA y_j + dB y_{j+1} + dC y_{j-1}). */
VK_API int  vk_get_lhs(vk_handle *h, double *jv, double *dA, double *dB, double *dC);

#ifdef __cplusplus
}
#endif
#endif /* VK_ROS2_H */
