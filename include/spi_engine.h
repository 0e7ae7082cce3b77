/*
 * spi_engine.h -- C ABI of the GB300 batched candidate-evaluation engine.
 *
 * Drop-in for the replay-evaluation path of SPI-Active. The reference
 * evaluates one parameter vector theta at a time across Isaac Gym envs; this
 * engine evaluates a batch of theta samples against a batch of logged windows
 * in one launch. Every call returns an int status (SPI_OK or a negative
 * SPI_E* code; spi_last_error() gives the message). Pointers documented as
 * "device" are CUDA device pointers owned by the caller (e.g. torch
 * data_ptr()); the engine never frees caller memory. An engine is bound to
 * one CUDA stream; calls are thread-compatible, not thread-safe.
 *
 * Reference interfaces replaced (paths inside the reference project):
 *   spi_create        <- scripts/eval.py:313-321 instantiate_env (env + sim creation)
 *   spi_load_windows  <- scripts/eval.py:174-182 to_device, plus the per-chunk reset of
 *                        evaluate_batch :243-277 (root state / dof state written from the window)
 *   spi_set_theta     <- scripts/eval.py:204-214 apply_base_mass and
 *                        spigym/simulator/isaacgym/isaacgym_active_sysid.py:39-95 set_<param>
 *   spi_run           <- scripts/eval.py:217-310 evaluate_batch (H x env.step, final-step
 *                        errors, masked sums, normaliser)
 *   spi_read_costs    <- the MassEvalResult of scripts/eval.py:38-42 / :306-310 and
 *                        scripts/mass_opt.py:62-76 compute_cost
 *   spi_run_trace     <- reading simulator.robot_root_states / dof_state after every
 *                        env.step (spigym/simulator/isaacgym/isaacgym.py:567-577)
 *   spi_cem_*         <- the Optuna ask/tell loop of scripts/mass_opt.py:203-219
 *                        (TPE there; CEM here, on the device)
 */
#ifndef SPI_ENGINE_H
#define SPI_ENGINE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPI_ABI_VERSION 1

#define SPI_OK 0
#define SPI_EINVAL (-1)      /* bad argument or size */
#define SPI_ENOMEM (-2)      /* device allocation failed */
#define SPI_ECUDA (-3)       /* CUDA runtime error */
#define SPI_ESTATE (-4)      /* call out of order (e.g. run before load) */
#define SPI_ETIMEOUT (-5)    /* reserved: no entry point waits on the device (no kernel spins) */
#define SPI_EBUDGET (-6)     /* request exceeds the admission budget */

#define SPI_STATE_DIM 37     /* pos3 quat4(xyzw) linvel3 angvel3 (world) q12 qd12 */
#define SPI_THETA_DIM 13
#define SPI_N_JOINTS 12
#define SPI_N_LEG_BODIES 12
#define SPI_N_COMP 9         /* |dp| |dquat| |dq| |dp|^2 |dquat|^2 |dv|^2 |dw|^2 |dq|^2 |dqd|^2 */

/* theta slots: 0 base mass [kg]; 1-3 base CoM offset [m]; 4 base inertia-diagonal scale;
 * 5-8 front legs (FL, FR): Kp scale, Coulomb friction [N m], armature [kg m^2], torque-limit
 * scale; 9-12 rear legs (RL, RR): the same four. */

/* Robot model and simulation settings. Leg bodies are ordered FL, FR, RL, RR x hip, thigh,
 * calf (the Isaac Gym DFS order of spigym/config/robot/go2/go2.yaml:29); hip joints rotate
 * about x, thigh and calf joints about y. Inertias are 6 floats xx yy zz xy xz yz.
 * The kernels take the Go2's joint-origin pattern: hip origins in the base's x-y plane,
 * thigh origins on the hip's y axis, calf origins on the thigh's z axis, the foot on the
 * calf's z axis. Every entry point that takes a spi_robot returns SPI_EINVAL for any other. */
typedef struct spi_robot {
    float body_origin[SPI_N_LEG_BODIES][3]; /* joint origin in the parent frame */
    float body_mass[SPI_N_LEG_BODIES];
    float body_h[SPI_N_LEG_BODIES][3];      /* mass * CoM (body frame) */
    float body_I[SPI_N_LEG_BODIES][6];      /* rotational inertia about the body origin */
    float base_mass_nominal;
    float base_com[3];                      /* nominal base CoM; theta[1:4] offsets it */
    float base_Ic[6];                       /* nominal base inertia about its CoM */
    float fixed_mass;                       /* collapsed fixed links on the base (heads) */
    float fixed_h[3];
    float fixed_I[6];                       /* about the base origin */
    float foot[3];                          /* foot contact point in the calf frame */
    float foot_radius;
    float corners[8][3];                    /* base collision-box corners (base frame) */
    float contact_k, contact_c, contact_ct, contact_mu;
    float contact_ramp;                     /* penetration over which the normal damping fades in [m] */
    float kp[SPI_N_JOINTS], kd[SPI_N_JOINTS];
    float kd_scale, action_scale, action_clip, hip_action_scale;
    float default_q[SPI_N_JOINTS], torque_limit[SPI_N_JOINTS], velocity_limit[SPI_N_JOINTS];
    float motor_gain[3];                    /* per joint type hip/thigh/calf, after the clip */
    float tanh_a[3];                        /* a*tanh(tau/a) per joint type; 0 disables */
    float friction_vel;                     /* Coulomb friction tanh width [rad/s] */
    float sim_dt;                           /* physics substep [s] */
    float gravity;
    int32_t decimation;                     /* substeps per control step */
    int32_t torque_speed;                   /* torque limit falls linearly to 0 at velocity_limit */
    int32_t base_contact;                   /* base box corners collide */
    int32_t inertia_follows_mass;           /* base inertia scales with mass/nominal */
} spi_robot;

typedef struct spi_engine spi_engine;

int spi_abi_version(void);
/* Message of the last failing call on this thread ("" if none). */
const char* spi_last_error(void);

int spi_create(const spi_robot* robot, spi_engine** out);
int spi_destroy(spi_engine* e);
/* Bind the engine to a cudaStream_t (NULL = legacy default stream). */
int spi_set_stream(spi_engine* e, void* stream);

/* Windows, device pointers in the reference's row layout: init and target [W][37] states,
 * actions [W][H][12] (raw policy actions, clipped and scaled inside), weight [W] per-window
 * weight (NULL = all 1), norm = divisor of the weighted sums (the reference's count of
 * non-end windows; <= 0 means W). Copied into engine-owned structure-of-arrays storage. */
int spi_load_windows(spi_engine* e, const float* init, const float* actions,
                     const float* target, const float* weight, int W, int H, float norm);

/* Theta batch, device [N][13]. Copied into engine storage. */
int spi_set_theta(spi_engine* e, const float* theta, int N);

/* Cost weights: mode 0 = reference L2 (10/5/1 on |dp|, |dquat|, |dq|; scripts/mass_opt.py:28-32),
 * mode 1 = weighted squared error with sq_weights[6] (pos, quat, linvel, angvel, q, qd). */
int spi_set_cost(spi_engine* e, int mode, const float* sq_weights);

/* Rollout-kernel variant: the register allocator targets min_blocks CTAs of 128 threads per
 * SM (2: 255 registers; 3: 168; 4: 128; 5: 96; the quad and block layouts take 3..5, the lane
 * layout 2..4, larger values act as 4). Same equations; results within FP32 rounding of each
 * other. */
int spi_set_kernel_config(spi_engine* e, int min_blocks);

/* Rollout-kernel lane layout (default after spi_create: SPI_LAYOUT_LANE with min_blocks 3).
 * SPI_LAYOUT_QUAD: four lanes per rollout, one leg each, the base
 * solved on all four. SPI_LAYOUT_LANE: one lane per rollout through all four legs, the model
 * in the kernel's parameter block, 68 KB of shared memory per 128-thread CTA (three CTAs per
 * SM); min_blocks 2..4 sets the register cap (4: 128 registers). Same equations, results
 * within FP32 rounding of each other; spi_run_trace always uses the quad layout. */
#define SPI_LAYOUT_QUAD 0
#define SPI_LAYOUT_LANE 1
/* SPI_LAYOUT_BLOCK: the quad layout with each rollout's base solved once per substep by one
 * warp of the CTA (one lane per rollout) instead of on all four of its lanes; two CTA
 * barriers per substep; min_blocks 3..5. */
#define SPI_LAYOUT_BLOCK 2
int spi_set_kernel_layout(spi_engine* e, int layout);

/* Roll every (theta, window) pair H control steps and reduce the windowed cost. Async. */
int spi_run(spi_engine* e);
/* Same, also writing every control step's state to trace, device [N][W][H][37]. */
int spi_run_trace(spi_engine* e, float* trace);

/* Advance caller-owned states in place: state device [B][37] (world frame, the reference's
 * root-state row + dof positions + dof velocities), actions device [B][steps][12], theta device
 * [B][13]. The simulator step of the reference (spigym/simulator/base_simulator/
 * base_simulator.py:121-150 under spigym/envs/legged_base_task/legged_robot_base.py:169-209).
 * Asynchronous on the engine stream. */
int spi_step_states(spi_engine* e, float* state, const float* actions, const float* theta, int B, int steps);

/* Copy results of the last run (async on the engine stream): comp device [N][9] mean
 * components (may be NULL), cost device [N] scalar cost (may be NULL). */
int spi_read_costs(spi_engine* e, float* comp, float* cost);

/* Copy the current theta batch [N][13] to theta (device or pinned host), async. */
int spi_read_theta(spi_engine* e, float* theta);

/* Wait for the engine stream; report the number of (theta, window) rollouts whose final state
 * was not finite, counted since spi_create. */
int spi_sync(spi_engine* e, int64_t* n_nonfinite);

/* ---- cross-entropy-method identification on the device -------------------------------
 * Replaces the host-side Optuna ask/tell loop of scripts/mass_opt.py:203-219 (TPE) and the
 * grid of scripts/mass_landscape.py:153 with a CEM whose sampling, elite selection, mean /
 * covariance refit and FP64 Cholesky run on the GPU. The engine's theta batch becomes the
 * CEM population; slots not identified keep their nominal value. */
typedef struct spi_cem_config {
    int32_t n_samples;                       /* population N (2 .. 16384) */
    int32_t dim;                             /* identified parameters P (1 .. 13) */
    int32_t param_ids[SPI_THETA_DIM];        /* theta slot of each identified parameter */
    float nominal[SPI_THETA_DIM];            /* values of the other slots */
    double lo[SPI_THETA_DIM], hi[SPI_THETA_DIM];  /* prior box per identified parameter */
    double elite_frac;                       /* elites = max(2, floor(elite_frac * N + 0.5)) */
    double alpha;                            /* smoothing of mean and covariance (1 = none) */
    double min_std_frac;                     /* per-dimension std floor, fraction of hi - lo */
    uint64_t seed;                           /* Philox4x32-10 key */
    int32_t job_id;                          /* Philox counter word 3 */
} spi_cem_config;

int spi_cem_init(spi_engine* e, const spi_cem_config* cfg);
/* Draw this iteration's population into the theta batch (iteration 0: uniform prior box). */
int spi_cem_sample(spi_engine* e);
/* Refit from the last run's costs; iteration += 1. */
int spi_cem_refit(spi_engine* e);
/* sample + run + refit, all asynchronous on the engine stream. */
int spi_cem_step(spi_engine* e);
/* `iterations` steps; with use_graph one step is captured once as a CUDA graph and replayed. */
int spi_cem_run(spi_engine* e, int iterations, int use_graph);
/* Synchronous read of the distribution (host pointers, any may be NULL): mu [P],
 * cov [P][P], best theta [13] and cost over all iterations, iterations done. */
int spi_cem_read(spi_engine* e, double* mu, double* cov, float* best_theta, float* best_cost,
                 int32_t* iteration);

/* ---- sensitivities and Fisher information (active excitation design) ------------------
 * Replaces the finite-difference Fisher proxy of the reference
 * (spigym/envs/sysid/active_sysid_openloop.py:402-426, main env vs aux envs with theta + 0.1,
 * trace(J^T J)) with exact forward-mode derivatives of the rollout.
 * spi_sensitivity: J[n][w][i][k] = d s_H[i] / d theta[param_ids[k]] of window w (the loaded
 * windows) for theta sample n (device [N][13]); J device [N][W][37][K]; xH device
 * [N][W][37] final states or NULL. K <= 13. Asynchronous on the engine stream.
 * spi_fisher: F[n] = sum_w J_w^T diag(state_weight) J_w (device [N][K][K], FP32
 * accumulation), logdet[n] = log det(F[n] + eps I) and trace[n] = trace(F[n]) in FP64
 * (device [N] each, may be NULL). */
int spi_sensitivity(spi_engine* e, const float* theta, int N, const int32_t* param_ids, int K, float* J,
                    float* xH);
int spi_fisher(const float* J, int N, int W, int K, const float* state_weight, double eps, float* F,
               double* logdet, double* trace, void* stream);
/* As spi_fisher; tensor_cores = 1 accumulates J^T Q J on the tensor cores (BF16 operands, FP32
 * accumulation, warp-level mma m16n8k16), 0 on the CUDA cores in FP32. */
int spi_fisher_ex(const float* J, int N, int W, int K, const float* state_weight, double eps, int tensor_cores,
                  float* F, double* logdet, double* trace, void* stream);

/* ---- gradient by the adjoint of the rollout ------------------------------------------------
 * The reference has no gradient: its active exploration differences a main env against aux envs
 * with theta + 0.1 (spigym/envs/sysid/active_sysid_openloop.py:402-426). spi_adjoint gives, for
 * theta device [N][13] against the loaded windows, cost[n] = the engine's cost (spi_set_cost
 * mode and weights, the window weights and normaliser of spi_load_windows) and grad[n][13] =
 * d cost[n] / d theta[n] by a hand-written reverse sweep of the rollout: the forward pass keeps
 * the state every 5 control steps, the reverse pass recomputes each 5-step segment forward and
 * runs the substep adjoints backwards through it. cost and grad are device pointers (either may
 * be NULL). Non-finite final states are counted as by spi_run (spi_sync). Asynchronous on the
 * engine stream. */
int spi_adjoint(spi_engine* e, const float* theta, int N, float* cost, float* grad);

/* ---- the device CEM over a caller-scored population ----------------------------------------
 * Replaces the Optuna ask / tell of the reference's excitation search
 * (spigym/agents/sysid/active_sysid.py:165-257; CmaEsSampler, spigym/config/algo/
 * active_sysid.yaml:20) for searches whose candidates are not scored by spi_run. The same
 * sampling and refit kernels as spi_cem_*: spi_search_sample draws a population [n][13] into a
 * buffer the search owns (the identified slots sampled, the others at cfg->nominal) and returns
 * its device address; spi_search_refit takes the caller's device costs [n] (lower is better).
 * All calls are asynchronous on `stream` except create and read. */
typedef struct spi_search spi_search;
int spi_search_create(const spi_cem_config* cfg, void* stream, spi_search** out);
int spi_search_destroy(spi_search* s);
int spi_search_sample(spi_search* s, float** population);
int spi_search_refit(spi_search* s, const float* cost);
/* Synchronous: mean [P], covariance [P][P], best candidate [13] and cost, iterations done. */
int spi_search_read(spi_search* s, double* mu, double* cov, float* best, float* best_cost, int32_t* iteration);

/* ---- the reference's finite-difference Fisher objective -------------------------------------
 * spi_fd_fisher runs the open-loop active-sysid episode of the reference for C candidate
 * excitations at once: spigym/envs/sysid/active_sysid_openloop.py:29-80 (each candidate is a
 * group of 1 main + P aux rollouts, aux k at theta + delta on slot param_ids[k]), :246-252 and
 * :316-330 (after 1-based control step t with t % ksync == 1, or after every step when
 * 0 <= ksync <= 1, the aux rollouts take the main's state; never when ksync < 0) and :402-426
 * (after every step the reward
 * trace(J^T J), J = (s_main - s_aux) / delta over the 13 root-state entries and 12 joint
 * positions). x0 device [C][37] start states, actions device [C][T][12], theta device [C][13]
 * (each group's main theta), param_ids host [P] (P <= 13, distinct slots). reward_sum device
 * [C] receives the reward summed over steps t > skip (1-based); reward_trace device [C][T] each
 * step's reward, or NULL. Asynchronous on the engine stream; the engine's windows and theta
 * batch are not used. */
int spi_fd_fisher(spi_engine* e, const float* x0, const float* actions, const float* theta, int C, int T,
                  const int32_t* param_ids, int P, float delta, int ksync, int skip, float* reward_sum,
                  float* reward_trace);

/* ---- continuous-batching identification server ------------------------------------------
 * Many sysid jobs of uneven population, window count, horizon and parameter dimension share
 * the GPU. Each job is one CEM identification (the work of scripts/mass_opt.py per dataset);
 * jobs are admitted into slots against an HBM budget as they arrive, every tick advances
 * every active job by one CEM iteration in one rollout launch (work items are (job, theta,
 * 8-window group), one warp each, laid out longest horizon first), and finished jobs free
 * their slot and memory for the next arrivals. One tick is captured once as a CUDA graph. A
 * job's results do not depend on the other jobs in the mix, and equal the single-job engine's
 * (spi_cem_*) bit for bit: the server and spi_run launch the same compiled rollout kernel.
 * No counterpart in the reference, which runs one job at a time. */
typedef struct spi_server spi_server;

typedef struct spi_job {
    const float* init;       /* device [W][37] */
    const float* actions;    /* device [W][H][12] */
    const float* target;     /* device [W][37] */
    const float* weight;     /* device [W] or NULL */
    int32_t W, H;
    float norm;              /* <= 0: W */
    int32_t iterations;      /* CEM iterations to run */
    spi_cem_config cem;      /* population, identified slots, priors, seed */
} spi_job;

typedef struct spi_job_result {
    int32_t job_id;          /* spi_cem_config.job_id of the job */
    int32_t iterations;
    float best_cost;
    float best_theta[SPI_THETA_DIM];
    double mu[SPI_THETA_DIM];            /* mean over the identified parameters (first `dim`) */
    int32_t dim;
    int32_t status;          /* 0 ok, 1 covariance needed the std floor at some refit */
} spi_job_result;

/* max_slots concurrent jobs, each with at most max_samples theta; hbm_budget_bytes caps the
 * device memory of admitted jobs (spi_server_job_bytes gives a job's share). */
int spi_server_create(const spi_robot* robot, int max_slots, int max_samples, size_t hbm_budget_bytes,
                      spi_server** out);
int spi_server_destroy(spi_server* s);
int spi_server_set_stream(spi_server* s, void* stream);
int spi_server_set_cost(spi_server* s, int mode, const float* sq_weights);
size_t spi_server_job_bytes(const spi_job* job);
/* Admit a job: SPI_OK and its slot, or SPI_EBUDGET when no slot or memory is free now. The
 * window buffers are copied; the caller may free them once the call returns. */
int spi_server_submit(spi_server* s, const spi_job* job, int32_t* slot);
/* One CEM iteration for every active job (asynchronous). */
int spi_server_tick(spi_server* s);
/* Collect up to `max` finished jobs (host results); *n_done receives how many. */
int spi_server_poll(spi_server* s, spi_job_result* results, int max, int32_t* n_done);
/* Block until every tick and result copy enqueued so far has finished. */
int spi_server_wait(spi_server* s);
/* Active job count and free budget. */
int spi_server_stats(spi_server* s, int32_t* active, size_t* bytes_free);
/* Cap on rollout work per tick, in work items (one theta x 8-window group in the quad layout,
 * four of them in the lane layout; 0 = no cap). Admission depends only on slots and
 * the HBM budget; each tick then runs the admitted jobs with the least remaining work
 * (remaining iterations x work items x horizon) first, as many as fit the cap (at least one),
 * and the others stay resident until they are among the shortest. Once the GPU is full,
 * running more jobs at once only slows each of them down; shortest-remaining-work order
 * lets a short job that arrives during a long one finish first. */
int spi_server_set_work_cap(spi_server* s, long long max_items);
/* Rollout-launch shape: ctas_per_sm > 0 caps a launch at that many CTAs per SM (each warp then
 * takes as many consecutive work items as the cap requires); 0 = one warp per claim, no cap.
 * items_per_claim: consecutive work items per warp (1 .. 64). */
int spi_server_config(spi_server* s, int ctas_per_sm, int items_per_claim);
/* Rollout-kernel occupancy variant (the launch-bounds CTAs per SM: 3 or 4 in the quad layout,
 * 2 to 4 in the lane layout), as spi_set_kernel_config. */
int spi_server_set_kernel_config(spi_server* s, int min_blocks);
/* Rollout-kernel lane layout of the server: SPI_LAYOUT_QUAD (min_blocks 3 or 4) or
 * SPI_LAYOUT_LANE (one lane per rollout, work items of four 8-window groups; min_blocks 2 to 4), as
 * spi_set_kernel_layout. Only while no job is held (SPI_ESTATE otherwise). */
int spi_server_set_kernel_layout(spi_server* s, int layout);
/* CEM-iteration rounds per tick (1..8, default 1). Each tick runs this many rounds of one
 * iteration (sample, rollout, finalize, refit); a job takes part in as many rounds as the
 * largest active job's work per iteration (work items x horizon) is a multiple of its own,
 * capped by its remaining iterations, so small jobs advance several iterations per tick. */
int spi_server_set_rounds(spi_server* s, int rounds);

/* ---- evaluation without any device allocation ---------------------------------------
 * No counterpart in the reference. For callers that must not let a library call cudaMalloc:
 * a serving process that reserves its HBM budget up front, a host framework that owns every
 * device allocation, or a loop where cudaMalloc's implicit device synchronisation would stall
 * other streams. Same dynamics and costs as spi_load_windows + spi_set_theta + spi_run +
 * spi_read_costs, but the caller's row-layout device buffers are read directly (init and
 * target [W][37], actions [W][H][12], weight [W] or NULL, theta [N][13]; outputs comp [N][9]
 * and cost [N], either may be NULL), the model is passed by value to the kernel, and the
 * per-(theta, 8-window group) partial sums use a fixed file-scope device array that every
 * GPU loading the library keeps until exit: N * ceil(W / 8) <= SPI_NOALLOC_MAX_GROUPS, larger
 * requests fail with SPI_EINVAL. All calls share that array, so calls that overlap on the GPU
 * race; serialise them. The first call on a device looks up the array's address on that
 * device; make it before any stream capture. Asynchronous on `stream` (a cudaStream_t).
 * Unlike spi_run, it counts no non-finite rollouts (there is no spi_sync counter behind it): a
 * rollout whose final state is not finite shows up as non-finite entries in that theta's row of
 * comp, so callers check comp (or cost) for NaN / inf themselves. */
#define SPI_NOALLOC_MAX_GROUPS 65536
int spi_eval_windows_noalloc(const spi_robot* robot, const float* init, const float* actions,
                             const float* target, const float* weight, int W, int H, float norm,
                             const float* theta, int N, int cost_mode, const float* sq_weights,
                             float* comp, float* cost, void* stream);

/* Upper bound of the FP32 throughput of this GPU, measured by an FMA loop [FLOP/s]. */
int spi_probe_fp32_peak(double* flops_per_s);

#ifdef __cplusplus
}
#endif
#endif /* SPI_ENGINE_H */
