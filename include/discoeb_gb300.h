/*
 * discoeb_gb300.h -- C ABI of the GB300 perturbation solver.
 *
 * Replaces, for one GPU, the hot path of the reference's
 *   discoeb.perturbations.evolve_perturbations   (src/discoeb/perturbations.py:926-997)
 * i.e. the vmap over k-modes of evolve_one_mode (perturbations.py:728-781):
 * start time + adiabatic ICs + Rodas5(transformed) + PID step control +
 * SaveAt linear interpolation + conversion to the 20 output fields.  The
 * get_power assembly (perturbations.py:1101-1123) is deb_get_power below.
 *
 * Conventions
 *   - every pointer named d_* is a caller-owned DEVICE buffer;
 *   - calls are stream-ordered on `stream` (a cudaStream_t passed as void*,
 *     NULL = legacy default stream) and do not synchronise the host, except
 *     deb_plan_create / deb_plan_destroy;
 *   - return value 0 = success, < 0 = deb_status error code (no exceptions
 *     cross the ABI); per-mode solver outcomes go to d_status;
 *   - a plan is not thread-safe: one plan per stream.
 *
 * Table blob (FP64, one per cosmology, all blobs of one call the same length)
 *   [0..31]   header: Omegam, Omegab, OmegaDE, Omegak, grhom, grhog, grhor,
 *             Neff, Nmnu, amnu, w_DE_0, w_DE_a, cs2_DE, YHe, H0, taumin, A_s,
 *             n_s, k_p, nq, n_spline[7], blob_len, magic (20231103),
 *             derived_offset, 0, 0
 *   splines   7 x (x[n], y[n], S[n]) in the order xe(log a), c_s^2 a(log a),
 *             log rho_nu(log a), log p_nu(log a), a(tau), tau(a), xe(tau)
 *             (fields _x_, _y_, _S_full_ of spline_interpolation.py:112-113)
 *   nodes     q[nq], w[nq] of get_neutrino_momentum_bins (background.py:13-44)
 *   derived   7 x (c[4(n-1)] polynomial coefficients of each interval,
 *             p(u) = c0 + u (c1 + u (c2 + u c3)), u = x - x_i; then the
 *             n knots as FP32, packed into ceil(n/2) doubles)
 */
#ifndef DISCOEB_GB300_H
#define DISCOEB_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DEB_HDR_LEN 32
#define DEB_TABLE_MAGIC 20231103.0
#define DEB_NOUT_FIELDS 20

/* error codes (return values) */
enum deb_status {
  DEB_OK = 0,
  DEB_ERR_INVALID = -1,     /* bad argument (sizes, NULL pointer, lmax < 3) */
  DEB_ERR_TABLES = -2,      /* table blob header / magic / sizes inconsistent */
  DEB_ERR_CUDA = -3,        /* a CUDA runtime call failed */
  DEB_ERR_NOMEM = -4,       /* device allocation for the plan failed */
  DEB_ERR_CAPACITY = -5,    /* more modes or variables than the plan was made for */
  DEB_ERR_STATIC_SCRATCH = -6 /* deb_forward_static: one mode's state exceeds DEB_STATIC_SCRATCH_BYTES */
};

/* per-mode outcome written to d_status (same meaning as the oracle's) */
enum deb_mode_status {
  DEB_MODE_OK = 0,
  DEB_MODE_MAX_STEPS = 1,   /* diffrax would raise: max_steps reached (perturbations.py:762) */
  DEB_MODE_DT_UNDERFLOW = 2,/* step size no longer advances tau */
  DEB_MODE_NONFINITE = 3,   /* NaN/Inf in the error estimate (e.g. w = -1 exactly) */
  DEB_MODE_BAD_INPUT = 4    /* k <= 0, cosmology index out of range, bad tables */
};

/* linear solver for W = I/(gamma h) - J */
enum deb_linear_solver {
  DEB_SOLVE_STRUCTURED = 0, /* exact block/chain elimination + rank-2 Woodbury, O(n) */
  DEB_SOLVE_DENSE = 1       /* dense LU with partial pivoting, O(n^3), as the reference */
};

/* how modes map onto the GPU */
enum deb_exec_mode {
  DEB_EXEC_AUTO = 0,        /* warp per mode for small batches, lane per mode for large ones */
  DEB_EXEC_LANE = 1,        /* one thread per mode, state interleaved in global memory */
  DEB_EXEC_WARP = 2         /* one warp per mode, state in shared memory */
};

/* hierarchy sizes: the keyword arguments of evolve_perturbations (perturbations.py:926-930) */
typedef struct deb_dims {
  int lmaxg, lmaxgp, lmaxr, lmaxnu, nqmax;
  int nout;            /* output times per cosmology */
  int return_full;     /* 0: 20 output fields, 1: full state of nvar entries */
  int linear_solver;   /* enum deb_linear_solver */
  int exec_mode;       /* enum deb_exec_mode */
} deb_dims;

/* PIDController arguments of evolve_one_mode (perturbations.py:759-760) plus
   diffrax defaults the reference inherits (safety 0.9, error order 5). */
typedef struct deb_solver_cfg {
  double rtol, atol;
  double pcoeff, icoeff, dcoeff;
  double factormax, factormin;
  double safety;
  double error_order;
  int max_steps;
  int hist_on_reject;  /* 1: a rejected step also shifts the error history */
  int step_to_outputs; /* 0: outputs by linear interpolation inside the step (the
                          reference's SaveAt(ts), perturbations.py:770); 1: steps
                          are clipped to land on every output time (diffrax
                          PIDController(step_ts=...)), outputs are step ends */
} deb_solver_cfg;

typedef struct deb_plan deb_plan;

/* number of ODE variables, perturbations.py:739 */
int deb_nvar(const deb_dims* dims);

/* Create a plan for up to max_modes modes per call.  Allocates the solver
   workspace on the current device; deb_forward itself allocates nothing. */
int deb_plan_create(const deb_dims* dims, int max_modes, deb_plan** plan);

/* Bytes of device workspace the plan holds. */
int deb_plan_workspace_bytes(const deb_plan* plan, size_t* bytes);

/*
 * Launch shape of the warp-per-mode kernel, no reference counterpart (the
 * reference's vmap has no launch shape).  A mode's state is 16 vectors of
 * nvar doubles plus a small block; the first 8 vectors and the block always
 * live in shared memory, the 8 Rodas5 stage vectors either there too
 * (DEB_STAGE_SHARED: 44 KB per mode at nvar 323, 5 modes per SM) or in an
 * L2-resident global array (DEB_STAGE_GLOBAL: 24 KB of shared memory per
 * mode, up to 8 modes per SM, each stage access an L2 round trip).
 * modes_per_sm caps the modes in flight per SM (0: as many as fit).  Which
 * shape is faster depends on the hierarchy sizes; discoeb_gb300.autotune
 * times the candidates and picks one.  deb_plan_create uses
 * {DEB_STAGE_AUTO, 0}: shared when two modes fit per SM, else global.
 */
enum deb_stage_vectors { DEB_STAGE_AUTO = 0, DEB_STAGE_SHARED = 1, DEB_STAGE_GLOBAL = 2,
                         DEB_STAGE_ALL_GLOBAL = 3 /* the whole mode state in global memory (large nvar) */ };
typedef struct deb_launch_cfg {
  int stage_vectors;   /* enum deb_stage_vectors */
  int modes_per_sm;    /* cap on modes in flight per SM, 0 = no cap */
} deb_launch_cfg;
int deb_plan_create_ex(const deb_dims* dims, int max_modes, const deb_launch_cfg* launch, deb_plan** plan);
/* The shape a plan resolved to, and its modes in flight (resident warps). */
int deb_plan_launch_info(const deb_plan* plan, deb_launch_cfg* launch, int* modes_in_flight);

/*
 * Scheduling hint, no reference counterpart.  The kernel hands modes to its
 * warps through a device-side queue; a launch ends when its last mode ends,
 * and step counts differ by 60x across k, so handing out the most expensive
 * modes first shortens the tail.  d_order [nmode] (device) must be a
 * permutation of 0 .. nmode-1: queue position q takes mode d_order[q].
 * Results do not depend on it.  The plan keeps the pointer (the array must
 * stay valid until every launch that reads it has finished) and applies it
 * to deb_forward / deb_forward_record launches with this nmode; NULL
 * restores index order.  deb_replay always orders its work by the recorded
 * step counts, most steps first.
 */
int deb_plan_set_order(deb_plan* plan, const int* d_order, int nmode);

/*
 * Integrate nmode k-modes (perturbations.py:980-987 for one cosmology; here
 * any number of cosmologies share one launch).
 *   d_tables        [ncosmo, blob_len] FP64 table blobs
 *   d_k             [nmode] wavenumbers in 1/Mpc
 *   d_cosmo_of_mode [nmode] cosmology index of each mode (NULL: all 0)
 *   d_tau_out       [ncosmo, nout] conformal output times (tau_of_a(aexp_out))
 *   d_y_out         [nmode, nout, 20] (or [nmode, nout, nvar] if return_full)
 *   d_status        [nmode] deb_mode_status
 *   d_steps         [nmode, 2] accepted, rejected step counts (may be NULL)
 */
int deb_forward(deb_plan* plan, const double* d_tables, int ncosmo, int blob_len, const double* d_k,
                const int* d_cosmo_of_mode, int nmode, const double* d_tau_out, const deb_solver_cfg* cfg,
                double* d_y_out, int* d_status, int* d_steps, void* stream);

/*
 * Frozen-step tangents (the gradient path, a jax.jacfwd over the solve in
 * the reference: notebooks' compute_matter_power, perturbations.py:765
 * DirectAdjoint).  diffrax's PID controller stops gradients through its step
 * factor, so jacfwd differentiates the solve on the nominal step sequence.
 * deb_forward_record is deb_forward that also stores, per mode, tau_start and
 * every accepted step's end time:
 *   d_record [nmode, rec_len] (rec_len >= max_steps + 1), d_nrec [nmode]
 *   (accepted steps, 0 for a failed mode).
 * deb_replay integrates nset table sets per cosmology (e.g. theta +- eps per
 * parameter) on those recorded steps, without step control, in one launch:
 *   d_tables [ncosmo * nset, blob_len] (set s of cosmology c at row c*nset+s)
 *   d_tau_out [ncosmo * nset, nout]
 *   d_y_out [nset * nmode, nout, 20|nvar], d_status [nset * nmode]
 * The last replayed step ends at the set's own final output time.  Needs a
 * plan in DEB_EXEC_WARP (or AUTO) made for >= nset * nmode modes.
 */
int deb_forward_record(deb_plan* plan, const double* d_tables, int ncosmo, int blob_len, const double* d_k,
                       const int* d_cosmo_of_mode, int nmode, const double* d_tau_out, const deb_solver_cfg* cfg,
                       double* d_y_out, int* d_status, int* d_steps, double* d_record, int rec_len, int* d_nrec,
                       void* stream);
int deb_replay(deb_plan* plan, const double* d_tables, int ncosmo, int nset, int blob_len, const double* d_k,
               const int* d_cosmo_of_mode, int nmode, const double* d_tau_out, const deb_solver_cfg* cfg,
               const double* d_record, int rec_len, const int* d_nrec, double* d_y_out, int* d_status, void* stream);

/*
 * deb_forward_record that also keeps checkpoints for deb_adjoint: the state
 * after every ck_stride-th accepted step (and the initial state), at most
 * ck_cap of them per mode -- when the slots fill up every other one is
 * dropped and the stride doubles, so a mode keeps between ck_cap / 2 and
 * ck_cap evenly spaced states (ck_cap even, >= 2).
 *   d_ckpt [nmode, ck_cap, nvar], d_ckstride [nmode] (the final stride)
 * With d_ckoff (and d_ckcap) the slots are laid out per mode instead: mode m
 * owns d_ckcap[m] slots (taken down to even, >= 2) from slot d_ckoff[m] of
 * the pool d_ckpt [sum of caps, nvar], so that modes with long step
 * sequences get room for a state after every step (stride 1: the adjoint
 * recomputes nothing) while short ones take little; ck_cap is then unused.
 * No counterpart in the reference (jax.jacfwd keeps no states).
 */
int deb_forward_record_ckpt(deb_plan* plan, const double* d_tables, int ncosmo, int blob_len, const double* d_k,
                            const int* d_cosmo_of_mode, int nmode, const double* d_tau_out, const deb_solver_cfg* cfg,
                            double* d_y_out, int* d_status, int* d_steps, double* d_record, int rec_len, int* d_nrec,
                            double* d_ckpt, int ck_cap, const long long* d_ckoff, const int* d_ckcap,
                            int* d_ckstride, void* stream);

/*
 * Discrete adjoint of the recorded solve: for a cotangent of the output
 * fields, d L / d theta of the nominal solve's frozen-step map -- the
 * derivative the reference takes with jax.jacfwd through diffrax, whose PID
 * controller stops gradients through the step factor (perturbations.py:765,
 * DirectAdjoint; notebooks' compute_matter_power).  The map is: tau_start
 * and the ICs of each parameter set, the recorded step ends scaled by
 * tau_start / nominal tau_start (steps clipped to an output follow that
 * output time, the last step ends at the last output time), the Rodas5
 * steps (ode_integrators_stiff.py:718-834), SaveAt linear interpolation and
 * the output fields (perturbations.py:374-523).  One reverse sweep per
 * (seed, mode) replaces the 2 npar perturbed solves of deb_replay.
 *
 * theta enters through the tables: npar parameters, each given by its
 * theta_p + eps_p and theta_p - eps_p table sets; the adjoint takes the
 * derivatives of every table-dependent quantity it meets (the RHS
 * coefficients at each stage point, the output conversion, tau_start, the
 * ICs, tau_out) as central differences over those sets, everything else
 * (the integration) exactly.  The log-a splines (x_e, c_s^2 a, log rho_nu,
 * log p_nu) are evaluated on each set's own knots.
 *
 * A plan from deb_plan_create_adjoint (structured solver, 20 output fields,
 * lmaxg, lmaxgp, lmaxr >= 5, nqmax <= 64, nout <= 64) serves deb_adjoint
 * only; seg_cap = the largest checkpoint stride it accepts (a mode whose
 * stride exceeds it gets DEB_MODE_BAD_INPUT), max_items >= nseed * nmode.
 *   d_tables      [ncosmo, blob_len] nominal tables (those of the record)
 *   d_tables_pm   [ncosmo * 2 npar, blob_len]: set 2p = +eps_p, 2p+1 = -eps_p
 *   d_eps         [ncosmo, npar]
 *   d_tau_out     [ncosmo, nout], d_tau_out_pm [ncosmo * 2 npar, nout]
 *   d_record, rec_len, d_nrec, d_ckpt, ck_cap, d_ckoff, d_ckstride: from
 *                 deb_forward_record_ckpt on d_tables (d_ckoff may be NULL)
 *   d_gy          [nseed, nmode, nout, 20] cotangents of the output fields
 *   d_gtheta      [nseed, nmode, npar] dL/dtheta per seed and mode (NaN for
 *                 a failed item)
 *   d_status      [nseed * nmode] deb_mode_status
 * No counterpart in the reference (its gradient is forward mode).
 */
int deb_plan_create_adjoint(const deb_dims* dims, int max_items, int seg_cap, deb_plan** plan);
int deb_adjoint(deb_plan* plan, const double* d_tables, const double* d_tables_pm, int ncosmo, int npar, int blob_len,
                const double* d_eps, const double* d_k, const int* d_cosmo_of_mode, int nmode,
                const double* d_tau_out, const double* d_tau_out_pm, const double* d_record, int rec_len,
                const int* d_nrec, const double* d_ckpt, int ck_cap, const long long* d_ckoff, const int* d_ckstride,
                const double* d_gy, int nseed, double* d_gtheta, int* d_status, void* stream);

/*
 * The reference's batched variant, evolve_perturbations_batched
 * (perturbations.py:1000-1061 with evolve_modes_batched :835-922 and
 * Rodas5Batched, ode_integrators_stiff.py:846-1010): groups of batch_size
 * consecutive modes start together at the smallest of their start times
 * (:786-803), take one step sequence, and the PID controller sees one error
 * norm, the RMS over the six filtered entries of every mode of the group
 * (rms_norm_filtered_batched, :690-694).  A grouped plan (batch_size 1..32;
 * structured solver, 20 output fields) serves deb_forward_grouped only; its
 * arguments mean what they mean for deb_forward, nmode must be a multiple of
 * batch_size and every group must lie in one cosmology (else the group's
 * modes get DEB_MODE_BAD_INPUT); step_to_outputs must be 0.  Every mode of a
 * group reports the group's status and step counts.
 */
int deb_plan_create_grouped(const deb_dims* dims, int max_modes, int batch_size, deb_plan** plan);
int deb_forward_grouped(deb_plan* plan, const double* d_tables, int ncosmo, int blob_len, const double* d_k,
                        const int* d_cosmo_of_mode, int nmode, const double* d_tau_out, const deb_solver_cfg* cfg,
                        double* d_y_out, int* d_status, int* d_steps, void* stream);

/*
 * get_power (perturbations.py:1101-1123):
 *   P[m, o] = 2 pi^2 A_s (k_m/k_p)^(n_s-1) k_m^-3 y[m, o, idx]^2
 * with A_s, n_s, k_p read from the mode's cosmology blob.
 *   d_y      [nmode, nout, stride]   d_P [nmode, nout]
 */
int deb_get_power(const double* d_tables, int ncosmo, int blob_len, const double* d_k, const int* d_cosmo_of_mode,
                  int nmode, int nout, const double* d_y, int stride, int idx, double* d_P, void* stream);

void deb_plan_destroy(deb_plan* plan);

/*
 * Observables on top of the perturbations (no plan needed; stream-ordered).
 *
 * deb_power_multipoles -- power_multipoles (perturbations.py:1202-1224):
 *   with A = sqrt(2 pi^2 A_s (k/k_p)^(n_s-1) k^-3), delta = A y[.,4],
 *   theta = A y[.,5] (theta / aH, so -f delta in linear theory):
 *   P0 = b^2 delta^2 - 2b/3 delta theta + theta^2/5, P2 = -4b/3 delta theta
 *   + 4/7 theta^2, P4 = 8/35 theta^2.  d_y [nmode, nout, stride]; outputs [nmode, nout].
 * deb_density_velocity -- the delta and theta amplitudes above for one output
 *   (perturbations.py:1188-1190); d_y [nmode, stride]; d_delta, d_theta [nmode].
 * deb_power_kaiser -- power_Kaiser's P(k, mu) = (b delta - mu^2 theta)^2
 *   (perturbations.py:1198); d_Pkmu [nmode, nmu].
 * deb_savgol_log -- get_power_smoothed's filter (perturbations.py:1148-1159,
 *   util.py:407-444): exp of the 'same' convolution of ln P (nrow rows of n
 *   points) with d_coeffs[window] (window odd), the first window/2 and last
 *   window/2 + 1 points of each row copied from the input.
 * deb_fftlog_phase -- get_xi_from_P's phase factors (perturbations.py:1088-1094):
 *   exp(2i (arg Gamma((1.5+ell)/2 + i t_p) - ln(pi) t_p)), t_p = pi p / L,
 *   L = ln(kmax/kmin), p = 0..nfreq-1, as interleaved (re, im) pairs.
 */
int deb_power_multipoles(const double* d_tables, int ncosmo, int blob_len, const double* d_k, const int* d_cosmo_of_mode,
                         int nmode, int nout, const double* d_y, int stride, double bias, double* d_P0, double* d_P2,
                         double* d_P4, void* stream);
int deb_density_velocity(const double* d_tables, int ncosmo, int blob_len, const double* d_k, const int* d_cosmo_of_mode,
                         int nmode, const double* d_y, int stride, double* d_delta, double* d_theta, void* stream);
int deb_power_kaiser(const double* d_delta, const double* d_theta, int nmode, const double* d_mu, int nmu, double bias,
                     double* d_Pkmu, void* stream);
int deb_savgol_log(const double* d_P, int nrow, int n, const double* d_coeffs, int window, double* d_out, void* stream);
int deb_fftlog_phase(int nfreq, double log_kmax_over_kmin, int ell, double* d_phase, void* stream);

/*
 * Allocation-free variant of deb_forward.  No counterpart in the reference.
 *
 * Some callers cannot allocate device memory at all -- for example code that
 * runs inside a host framework which owns every device buffer and passes them
 * in (an XLA custom call, a serving process with a fixed memory pool).  They
 * cannot create a plan, because deb_plan_create calls cudaMalloc.  This entry
 * point needs no plan and allocates nothing: its scratch (the work-queue
 * counter and the per-mode solver state) lives in one fixed array of
 * DEB_STATIC_SCRATCH_BYTES compiled into the library, which every GPU that
 * loads the library holds until the process exits.  The caller still passes
 * all inputs and outputs, with the same meaning as for deb_forward.
 *
 *   - structured solver only (dims->linear_solver must be
 *     DEB_SOLVE_STRUCTURED); one warp per mode with its state in the array;
 *   - modes in flight are limited by the array (e.g. 380 at nvar 323, 1376 at
 *     nvar 80); any nmode is processed through the work queue;
 *   - returns DEB_ERR_STATIC_SCRATCH when one mode's state does not fit the
 *     array;
 *   - every call looks up the array's device address in the current context
 *     (cudaGetSymbolAddress); the first call in a context also uploads the
 *     constant tables (a synchronous copy): make that first call before any
 *     stream capture;
 *   - every call reuses the same array and resets the counter it needs, so
 *     calls that overlap on the GPU (e.g. on two streams) race: serialise them.
 */
#define DEB_STATIC_SCRATCH_BYTES (16u << 20)
int deb_forward_static(const deb_dims* dims, const double* d_tables, int ncosmo, int blob_len, const double* d_k,
                       const int* d_cosmo_of_mode, int nmode, const double* d_tau_out, const deb_solver_cfg* cfg,
                       double* d_y_out, int* d_status, int* d_steps, void* stream);

/*
 * Input tables on the GPU: the RECFAST branch of evolve_background
 * (background.py:140-342 with thermodynamics_recfast.py:124-501) for nset
 * parameter sets at once, written straight into table blobs.  One warp per
 * set; the adaptive GRK4A ionisation history runs on one lane, the sampled
 * quantities (neutrino tables, Saha fractions, sound speed, Romberg tau
 * integrals, spline coefficients) on all 32.
 *
 *   d_params [nset, DEB_BG_NPARAM]   input parameters in the order below
 *   d_consts [DEB_TC_COUNT]          RECFAST physical constants, fitting
 *                                    parameters and GRK4A coefficients (the
 *                                    host passes the numbers its own
 *                                    producer uses, so both agree)
 *   d_grid   parameter-independent grids, concatenated:
 *            a_nu[num_nu], log a_nu[num_nu] (neutrino tables),
 *            q[nq_bg], w[nq_bg] (their momentum quadrature),
 *            q[nqmax], w[nqmax] (the perturbations' momentum bins),
 *            a_thermo[num_thermo + 1] (RECFAST sampling), log a_thermo[1:]
 *   d_tables [nset, blob_len] output blobs, blob_len = deb_tables_blob_len()
 *   d_status [nset] (may be NULL): DEB_BG_* bits, 0 = ok
 */
enum deb_bg_status {
  DEB_BG_STEPS = 1,        /* an interval's step budget ran out (or a replayed step gave NaN) */
  DEB_BG_UNRECORDED = 2,   /* frozen form: the leader's step record overflowed step_cap; the
                              intervals past it ran adaptive */
  DEB_BG_BAD_LEADER = 4    /* frozen form: leader index out of range or itself a follower; ran adaptive */
};
enum deb_bg_param {
  DEB_BG_OMEGAM = 0, DEB_BG_OMEGAB, DEB_BG_H0, DEB_BG_TCMB, DEB_BG_YHE, DEB_BG_NEFF, DEB_BG_NMNU, DEB_BG_MNU,
  DEB_BG_W0, DEB_BG_WA, DEB_BG_CS2DE, DEB_BG_AS, DEB_BG_NS, DEB_BG_KP, DEB_BG_OMEGAK, DEB_BG_NPARAM
};
enum deb_tables_const {
  DEB_TC_G_N = 0, DEB_TC_MH, DEB_TC_ME, DEB_TC_MHE_MH, DEB_TC_C, DEB_TC_H_PLANCK, DEB_TC_KB, DEB_TC_BIG_H,
  DEB_TC_DENS_FAC, DEB_TC_E_ION_HE12S, DEB_TC_LAMBDA_H, DEB_TC_LAMBDA_HE, DEB_TC_L_HE1_ION, DEB_TC_L_HE_2P,
  DEB_TC_A2P_S, DEB_TC_A2P_T, DEB_TC_L_HE_2PT, DEB_TC_SIGMA_HE_2PS, DEB_TC_SIGMA_HE_2PT, DEB_TC_AGAUSS1,
  DEB_TC_AGAUSS2, DEB_TC_ZGAUSS1, DEB_TC_ZGAUSS2, DEB_TC_WGAUSS1, DEB_TC_WGAUSS2, DEB_TC_H_FRAC, DEB_TC_CDB,
  DEB_TC_CDB_HE, DEB_TC_CB1, DEB_TC_CR, DEB_TC_CK, DEB_TC_CK_HE, DEB_TC_CL, DEB_TC_CL_HE, DEB_TC_CT, DEB_TC_BFACT,
  DEB_TC_CL_PST, DEB_TC_HCL_HE2ST_KB, DEB_TC_HCL_HE2ST_ION_KB, DEB_TC_A_PPB, DEB_TC_B_PPB, DEB_TC_C_PPB,
  DEB_TC_D_PPB, DEB_TC_A_VF, DEB_TC_B_VF, DEB_TC_T0, DEB_TC_T1, DEB_TC_A_TRIP, DEB_TC_B_TRIP, DEB_TC_FU,
  DEB_TC_G, DEB_TC_G21, DEB_TC_G31, DEB_TC_G32, DEB_TC_G41, DEB_TC_G42, DEB_TC_G43, DEB_TC_A21, DEB_TC_A31,
  DEB_TC_A32, DEB_TC_CH1, DEB_TC_CH2, DEB_TC_CH3, DEB_TC_C1, DEB_TC_C2, DEB_TC_C3, DEB_TC_C4, DEB_TC_PI,
  DEB_TC_SQRT_PI, DEB_TC_C2OK, DEB_TC_COUNT
};
typedef struct deb_bg_cfg {
  int num_thermo;   /* RECFAST samples (evolve_background's num_thermo, 256) */
  int num_nu;       /* neutrino table points (512) */
  int nq_bg;        /* momentum bins of the background neutrino sums (8) */
  int nqmax;        /* momentum bins written into the blob for the perturbations */
  int max_steps;    /* GRK4A steps per sampling interval (128) */
  double amin;      /* 1e-9: taumin = amin / adotrad */
  double rtol, atol;/* GRK4A tolerances (1e-3, 1e-6) */
} deb_bg_cfg;
int deb_tables_blob_len(int num_thermo, int num_nu, int nqmax);
int deb_evolve_background(const deb_bg_cfg* cfg, const double* d_params, int nset, const double* d_consts,
                          const double* d_grid, double* d_tables, int blob_len, int* d_status, void* stream);
/* The same producer on the host cores (same code, compiled for the CPU): HOST
   buffers, nthreads worker threads over the sets (<= 0: one per hardware
   thread).  A RECFAST history is one long sequential chain of small FP64
   steps, which a CPU core runs far faster than one GPU lane; for a few
   hundred sets this is the faster producer. */
int deb_evolve_background_host(const deb_bg_cfg* cfg, const double* params, int nset, const double* consts,
                               const double* grid, double* tables, int blob_len, int* status, int nthreads);
/*
 * Frozen step sequences for difference quotients over parameter sets.  Set
 * s with leader[s] = -1 integrates its ionisation history adaptively and
 * records every accepted GRK4A step end, the case of the thermal history it
 * took in each interval and the branches of every RHS evaluation; a set with
 * leader[s] = j >= 0 (j a set with leader[j] = -1) takes set j's cases,
 * steps and branches instead, all steps accepted,
 * so that its tables are a smooth function of its parameters near set j's:
 * the derivative the reference's jax.jacfwd takes through its RECFAST
 * diffeqsolve (thermodynamics_recfast.py:283-298, forward mode through the
 * nominal step sequence and the branches the nominal values select).  Sets
 * with leader -1 give the same blobs as deb_evolve_background.
 *
 *   d_leader [nset]                                    device ints
 *   d_steps  [nset, 3 num_thermo + 1 + 2 step_cap]     scratch: per leader
 *            the first step of each interval, the case of each interval, the
 *            branch word of its closing RHS evaluation, then an (end, branch
 *            word) pair per step, all as doubles; follower rows are unused.
 *            step_cap = 16 num_thermo is ample at rtol 1e-3
 *            (DEB_BG_UNRECORDED reports an overflow).
 *
 * Two launches on `stream`: the leaders, then the followers.
 */
int deb_evolve_background_frozen(const deb_bg_cfg* cfg, const double* d_params, int nset, const int* d_leader,
                                 const double* d_consts, const double* d_grid, double* d_steps, int step_cap,
                                 double* d_tables, int blob_len, int* d_status, void* stream);
/* The frozen form on the host cores: HOST buffers; steps may be NULL (the
   library then keeps step_cap = 16 num_thermo per set itself). */
int deb_evolve_background_frozen_host(const deb_bg_cfg* cfg, const double* params, int nset, const int* leader,
                                      const double* consts, const double* grid, double* steps, int step_cap,
                                      double* tables, int blob_len, int* status, int nthreads);
/* tau_of_a (perturbations.py:975) of each blob at nout scale factors: d_tau [nset, nout] */
int deb_tau_of_a(const double* d_tables, int nset, int blob_len, const double* d_aexp, int nout, double* d_tau,
                 void* stream);

/* Measured-peak helper for roofline reporting: runs independent FP64 FMA
   chains on every SM and returns the achieved FP64 FLOP/s (FMA = 2).
   Allocates and frees 8 bytes of device memory and synchronises `stream`. */
int deb_measure_fp64_peak(double* flops_per_s, void* stream);

const char* deb_error_string(int code);
int deb_version(void);

#ifdef __cplusplus
}
#endif
#endif /* DISCOEB_GB300_H */
