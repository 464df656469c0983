// Device state of the batched integration loop (see vk_control.cu).
#pragma once
#include "vk_internal.cuh"

namespace vk {

struct RunState {
    double *y, *ymix, *y_prev;          // [L][ni]
    double *atm;                        // [L][VK_ATM_NF], same storage as DevBatch::atm
    double *dt, *t, *delta, *longdy, *longdydt;   // [ncols]
    double *aflux_change;               // [ncols] last radiative-transfer flux change (0: none)
    int *count, *end_case, *active, *natt, *steps_call, *pref;  // [ncols]
    int *counters;                      // [ncols][VK_NCOUNTERS]
    double *atom_ini, *loss, *loss_prev;  // [ncols][VK_MAX_NATOM]
    double *hist_y;                     // [conv_step][L][ni] ring of accepted states
    double *hist_t;                     // [ncols][conv_step]
    int *ignore;                        // [max_cols][ni]
};

struct RunCtrl {
    double rtol, atol, mtol, mtol_conv, pos_cut, nega_cut, loss_eps;
    double dt_min, dt_max, dt_var_min, dt_var_max;
    double yconv_cri, slope_cri, yconv_min, st_factor, trun_min, runtime;
    double gs, Rp, flux_cri;
    int conv_step, count_min, count_max, update_frq, max_attempts, flags, max_steps;
};

void launch_start(const DevNet &net, const DevBatch &b, const RunState &rs, const RunCtrl &cc,
                  cudaStream_t s);
void launch_control(const DevNet &net, const DevBatch &b, const RunState &rs, const RunCtrl &cc,
                    const double *sol, const double *ymix_sol, const double *delta,
                    const int *status, const int *fallback, double *geo, cudaStream_t s);
void launch_count_active(const int *active, int ncols, int *nactive, cudaStream_t s);
void launch_reset_columns(const RunState &rs, int n, const int *cols, double *dt, int *status,
                          double *thr64, double route_dt0, cudaStream_t s);

}  // namespace vk
