/*
 * gbdmc.h -- C ABI of the GB300 diffusion Monte Carlo walker-step library
 * (libgbdmc.so, sm_103a).
 *
 * Conventions
 *  - Every pointer named *_dev is device memory owned by the caller; the
 *    library allocates nothing on any call.  Host structs are read during the
 *    call only.
 *  - Walker arrays are structure-of-arrays: coordinate component k = 3*atom+dim
 *    of walker i lives at x[k*ld + i]; ld (leading dimension) >= capacity.
 *  - `stream` is a cudaStream_t passed as void* (NULL = legacy default stream).
 *  - Every call returns GBDMC_OK (0) or an error code; gbdmc_last_error()
 *    gives a message for the calling thread's last failure.
 *  - Calls are stream-ordered and asynchronous.  Population-control guards
 *    raised on the device are reported in gbdmc_ctrl_t.status, which the host
 *    reads once per batch of steps.
 *
 * The entry points replace the reference's plug-in and engine interfaces
 * (paths relative to the reference project root):
 *   gbdmc_pes_eval      <- Potential*.getpot(cds)          simulation_utilities/potential_manager.py:71,144,196,237
 *   gbdmc_trial_eval    <- ImpSamp.drift(cds) = call_trial + call_derivs
 *                          simulation_utilities/imp_samp.py:21-26, imp_samp_manager.py:92-139,197-224
 *   gbdmc_sim_init      <- DMC_Sim.propagate step-0 potential + calc_vref   pyvibdmc.py:760-769
 *   gbdmc_sim_step      <- one iteration of DMC_Sim.propagate               pyvibdmc.py:710-848
 *                          (move_randomly :540, imp_move_randomly :549, getpot :785-793,
 *                           local_kin :807-809, birth_or_death :380-454, calc_vref :651-661,
 *                           update_sim_arrays :674-682)
 *   gbdmc_desc_weights  <- DMC_Sim.calc_desc_wts                            pyvibdmc.py:663-672
 */
#ifndef GBDMC_H
#define GBDMC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBDMC_MAX_ATOMS 8
#define GBDMC_ABI_VERSION 1

/* return codes */
enum {
  GBDMC_OK = 0,
  GBDMC_ERR_ARG = 1,      /* invalid argument (sizes, kinds, null pointers) */
  GBDMC_ERR_CUDA = 2,     /* a CUDA runtime call failed */
  GBDMC_ERR_CAPACITY = 3  /* request exceeds a documented maximum */
};

/* device status bits (gbdmc_ctrl_t.status); any bit stops further steps */
enum {
  GBDMC_ST_NONFINITE_WEIGHT = 1, /* pyvibdmc.py:397 non-finite weight          */
  GBDMC_ST_HUGE_WEIGHT = 2,      /* pyvibdmc.py:397 weight > 1.5 N0 + 1        */
  GBDMC_ST_POP_LOW = 4,          /* pyvibdmc.py:409,716 population < 0.5 N0    */
  GBDMC_ST_POP_HIGH = 8,         /* pyvibdmc.py:409,716 population > 1.5 N0    */
  GBDMC_ST_OVERFLOW = 16,        /* population would exceed the capacity ld    */
  GBDMC_ST_TIMEOUT = 32          /* a bounded wait inside a kernel gave up     */
};

/* potential energy surfaces */
enum {
  GBDMC_PES_HO = 1,     /* p[0]=k : V = 1/2 k |x|^2                              */
  GBDMC_PES_H2O_LM = 2, /* O,H,H; p = De, a, re, ktheta, theta_e, krr            */
  GBDMC_PES_DIMER = 3,  /* O,H,H,O,H,H; p = De,a,re,ktheta,theta_e,krr,eps,sigma,qH,qO */
  GBDMC_PES_H2O_PS = 4, /* Partridge-Schwenke water (J. Chem. Phys. 106, 4618 (1997)), the reference's
                           sample Fortran PES (h2opes_v2.f).  p[0] = 0: atoms O,H,H; p[0] = 1: H,H,O (the
                           order of the reference's calc_hoh_pot, calc_h2o_pot.f:1-30)            */
  GBDMC_PES_EXTERNAL = 5 /* the caller's potential (any getpot, potential_manager.py:71-253): a step is
                           gbdmc_sim_move, the caller's V written to dst->v, then gbdmc_sim_branch.
                           p[0] = coordinates per walker nc (1..3*natoms; 0: 3*natoms), p[1] = dimensions
                           per atom d (1, 2 or 3; 0: 3).  Walker arrays keep 3*natoms rows, of which the
                           first nc are coordinate k = d*atom + dim and the rest padding; sigma[] is per
                           atom of the caller's system (nc / d atoms, at most GBDMC_MAX_ATOMS).      */
};

typedef struct {
  int32_t kind;
  int32_t natoms;
  double p[16];
} gbdmc_pes_t;

/* trial wave functions for importance sampling */
enum {
  GBDMC_TRIAL_NONE = 0,
  GBDMC_TRIAL_HO_GAUSS = 1,  /* p[a] = alpha of atom a; separable Cartesian Gaussian        */
  GBDMC_TRIAL_H2O_GAUSS = 2, /* O,H,H; p = alpha_r1, alpha_r2, alpha_th, r1e, r2e, theta_e  */
  GBDMC_TRIAL_DIMER_GAUSS = 3 /* O,H,H,O,H,H: the H2O trial of each monomer times a Gaussian in
                                 R_OO; p = the six H2O parameters, alpha_R, R_e                */
};

typedef struct {
  int32_t kind;
  int32_t natoms;
  double p[16];
} gbdmc_trial_t;

/* noise sources */
enum {
  GBDMC_NOISE_PHILOX32 = 0, /* Philox4x32-10, Box-Muller in fp32, widened to fp64 */
  GBDMC_NOISE_PHILOX64 = 1, /* Philox4x32-10, Box-Muller in fp64                  */
  GBDMC_NOISE_INJECTED = 2  /* caller-provided standard normals and uniforms      */
};

enum { GBDMC_DISCRETE = 0, GBDMC_CONTINUOUS = 1 };

/* walker state, SoA, caller-owned device memory.
 * Logical walker j of a replica with slot offset `off` is stored at slot
 * off + idx[off + j] when idx != NULL (lazy compaction after branching) and
 * at slot off + j when idx == NULL. */
typedef struct {
  double* x;    /* [3A][ld] coordinates (bohr)                               */
  double* v;    /* [ld] potential, or local energy when importance sampling */
  int32_t* who; /* [ld] ancestor index for descendant weighting, or NULL    */
  double* f;    /* [3A][ld] drift dpsi/dx / psi (importance sampling)       */
  double* psi;  /* [ld] trial psi (importance sampling)                     */
  double* ke;   /* [ld] local kinetic energy (importance sampling)          */
  double* w;    /* [ld] continuous weights, or NULL                         */
  int32_t* idx; /* [ld] gather index of the logical walkers, or NULL        */
  uint64_t* key; /* [ld] lineage keys of gbdmc_sim_run's Philox streams, or
                    NULL (then a launch takes the logical indices); read at a
                    launch's start and written with its output            */
} gbdmc_walkers_t;

/* device-resident control block (caller allocates sizeof(gbdmc_ctrl_t)) */
typedef struct {
  int64_t n;        /* population of the current walker buffer          */
  int64_t n_prev;   /* population before the last branching             */
  int64_t step;     /* index of the next step                           */
  double vref;      /* current reference energy                         */
  double dt_eff;    /* importance sampling: dt * accepted fraction      */
  double eff_ts;    /* importance sampling: cumulative effective time   */
  int32_t status;   /* GBDMC_ST_* bits; nonzero stops all further steps */
  int32_t err_step; /* step at which status was first raised            */
  uint32_t ticket;  /* last-block election counter (kept at 0 between calls) */
  int32_t flags;    /* guard bits raised by blocks of the running kernel; folded
                       into status by the kernel's last block */
  int64_t n_acc;    /* importance sampling: accepted moves, last step   */
  int64_t reserved[6];
} gbdmc_ctrl_t;

/* per-step history written by the device (each pointer may be NULL) */
typedef struct {
  double* vref;      /* [len] vref after step t        (pyvibdmc.py:678)  */
  double* pop;       /* [len] population or sum of weights (:680-682)     */
  int32_t* births;   /* [len] discrete births / continuous branched count */
  int32_t* deaths;   /* [len] discrete deaths                              */
  int32_t* rejected; /* [len] Metropolis rejections                        */
  double* vmin;      /* [len] min / max / mean potential before branching */
  double* vmax;
  double* vmean;
  double* eff_ts;    /* [len] cumulative effective time (importance sampling) */
  int64_t len;
} gbdmc_history_t;

typedef struct {
  int32_t natoms;
  int32_t weighting;   /* GBDMC_DISCRETE / GBDMC_CONTINUOUS */
  int32_t noise_mode;  /* GBDMC_NOISE_* */
  int32_t track_who;   /* gather ancestor ids with the walkers */
  int64_t ld;          /* capacity and leading dimension */
  int64_t n0;          /* target population num_walkers */
  double dt;
  double alpha;        /* 1/(2 dt) unless overridden (pyvibdmc.py:200-203) */
  double sigma[GBDMC_MAX_ATOMS];    /* sqrt(dt/m_a) (pyvibdmc.py:199) */
  double inv_mass[GBDMC_MAX_ATOMS];
  double thresh_lower; /* continuous weighting thresholds (pyvibdmc.py:214-231) */
  double thresh_upper; /* <= 0 : none */
  uint64_t seed;
  int32_t block_threads; /* walkers per tile / threads per block (32..256, multiple of 32);
                            0 = chosen from n0 so that the tiles spread over all SMs */
  uint32_t replica_id;   /* Philox stream of a single simulation (gbdmc_sim_*)      */
  gbdmc_pes_t pes;
  gbdmc_trial_t trial; /* kind GBDMC_TRIAL_NONE: plain DMC */
  gbdmc_history_t hist;
} gbdmc_sim_t;

/* One replica of a batched ensemble: its walkers occupy slots
 * [off, off + cap) of every SoA array of the batch.  The ranges of one
 * batch must not overlap and must lie inside [0, sim->ld). */
#define GBDMC_MAX_REPLICAS 64
typedef struct {
  int64_t off;     /* first slot                                    */
  int64_t cap;     /* slots reserved (>= 1.5 n0 + 1)                */
  int64_t n0;      /* target population num_walkers                 */
  uint32_t stream; /* Philox stream id of the replica               */
  int32_t reserved;
} gbdmc_replica_t;

/* injected noise for one step (GBDMC_NOISE_INJECTED only; device pointers) */
typedef struct {
  const double* normal;   /* [3A][ld_noise] standard normals for the move     */
  const double* u_branch; /* [ld_noise] uniforms for birth/death              */
  const double* u_accept; /* [ld_noise] uniforms for the Metropolis test      */
  int64_t ld_noise;
} gbdmc_noise_t;

/* library information */
int gbdmc_abi_version(void);
const char* gbdmc_last_error(void);

/* Bytes of device scratch the step calls need for capacity ld (block partials). */
size_t gbdmc_scratch_bytes(int64_t ld);

/* V(x) for n walkers; grad_dev (SoA like x, may be NULL) receives dV/dx.
 * n = 0 reads and writes nothing (the buffers may then be NULL). */
int gbdmc_pes_eval(const gbdmc_pes_t* pes, const double* x_dev, int64_t n, int64_t ld,
                   double* v_dev, double* grad_dev, void* stream);

/* psi, (dpsi/dx)/psi and (d2psi/dx2)/psi per Cartesian component.
 * n = 0 reads and writes nothing (the buffers may then be NULL). */
int gbdmc_trial_eval(const gbdmc_trial_t* trial, const double* x_dev, int64_t n, int64_t ld,
                     double* psi_dev, double* d1_dev, double* d2_dev, void* stream);

/* Step 0: potential (+ local KE) of the start walkers and the first vref.
 * ctrl->n must hold the start population; resets step, status, eff_ts. */
int gbdmc_sim_init(const gbdmc_sim_t* sim, const gbdmc_walkers_t* w, gbdmc_ctrl_t* ctrl_dev,
                   void* scratch_dev, void* stream);

/* One full walker step.  Reads the logical walkers of `src` (state + its
 * gather index) and writes the moved walkers in pre-branch order to the
 * state arrays of `dst`; with discrete weighting the branched population
 * is dst's state gathered through dst->idx (written by the call), with
 * continuous weighting dst->idx must be NULL and dst holds the walkers in
 * order.  src and dst must not share arrays.  noise may be NULL unless
 * sim->noise_mode == GBDMC_NOISE_INJECTED (normals/uniforms indexed by the
 * logical walker). */
int gbdmc_sim_step(const gbdmc_sim_t* sim, const gbdmc_walkers_t* src, const gbdmc_walkers_t* dst,
                   gbdmc_ctrl_t* ctrl_dev, void* scratch_dev, const gbdmc_noise_t* noise,
                   void* stream);

/* Up to max_steps steps of plain DMC in one launch, stopping before step
 * step_end: the loop of DMC_Sim.propagate (pyvibdmc.py:710-876) between two
 * events, for discrete weighting, Philox deviates and a built-in potential.
 * Each block holds a run of the population (in logical order) in shared
 * memory and keeps its walkers' copies there; a reducer warp per block
 * exchanges the blocks' sums of a step (vref, N', every block's count)
 * through one grid barrier while the block's other warps move the next step.
 * When the largest block's run would take more warps than an even split plus
 * one, or a block's copies do not fit its buffer, the walkers are split
 * evenly again through dst and a second grid barrier.  Waits are bounded
 * (GBDMC_ST_TIMEOUT on expiry).
 * The algorithm is gbdmc_sim_step's; the noise differs: a walker draws its
 * deviates and branching uniform from the Philox stream of its lineage key
 * (src->key, or its logical index when src->key is NULL; copy 0 keeps its
 * parent's key, copy r >= 1 of a walker with key k branching at step s takes
 * the SplitMix64 finaliser of k + r * 0x9E3779B97F4A7C15 + s *
 * 0xD1B54A32D192ED03), not of its logical index at every step; dst->key
 * (when not NULL) receives the keys with the walkers, so a walk split over
 * several launches is the walk of one.  src holds the ctrl->n compact walkers (idx NULL);
 * dst receives the compact walkers after the last step run (x, v, who), or
 * the moved unbranched walkers of a step whose guards tripped, or -- when no
 * step runs (status set, step >= step_end) -- a copy of src, so a queue of
 * calls alternating two buffers always leaves the walkers in the last call's
 * dst.  ctrl->step tells how far a launch got (a launch runs at most 2^30 /
 * blocks steps).  Scratch: gbdmc_sim_run_scratch_bytes(sim->ld), zeroed before
 * the first call (the kernel leaves its barrier words zeroed).  Returns
 * GBDMC_ERR_CAPACITY, before any launch, when the per-block buffers of
 * sim->n0 walkers do not fit shared memory. */
size_t gbdmc_sim_run_scratch_bytes(int64_t ld);
/* The multi-step kernel's noise of n walkers with lineage keys keys_dev at
 * step `step` (sim's seed, replica_id and noise mode, which must be a Philox
 * mode; 1, 3 or 6 atoms): normal_dev [3A][ld_noise] and u_dev [n], in the
 * layout of gbdmc_noise_t, so that gbdmc_sim_step on this injected noise
 * follows gbdmc_sim_run's walk step by step. */
int gbdmc_lineage_noise(const gbdmc_sim_t* sim, const uint64_t* keys_dev, int64_t n, int64_t step,
                        double* normal_dev, int64_t ld_noise, double* u_dev, void* stream);
int gbdmc_sim_run(const gbdmc_sim_t* sim, const gbdmc_walkers_t* src, const gbdmc_walkers_t* dst,
                  gbdmc_ctrl_t* ctrl_dev, void* scratch_dev, int64_t step_end, int32_t max_steps, void* stream);

/* Walkers in (page-locked) host memory for gbdmc_sim_run_host, in the SoA
 * layout of gbdmc_walkers_t with leading dimension ld >= sim->ld. */
typedef struct {
  double* x;     /* [3A][ld] coordinates (bohr)                        */
  double* v;     /* [ld] potentials (written), or NULL                 */
  int32_t* who;  /* [ld] ancestor ids, or NULL (needed when tracked)  */
  uint64_t* key; /* [ld] lineage keys, or NULL (logical indices)      */
  int64_t ld;
} gbdmc_host_walkers_t;

/* gbdmc_sim_run on walkers that live in host memory between calls, as the
 * reference's NumPy walker arrays do (propagate, pyvibdmc.py:701-876).
 * The host arrays must be page-locked (cudaHostAlloc / cudaHostRegister:
 * the device reads and writes them over the host link).  ctrl_host holds the
 * control block as the previous call (or, after gbdmc_sim_init, a copy of
 * ctrl_dev) left it; it must be page-locked too.  One call:
 *   1. the ctrl_host->n walkers of host (x, who, key) are the launch's input:
 *      read in place when host->ld == sim->ld, else copied into dev_src;
 *   2. gbdmc_sim_run(sim, input, dev_dst, ...) runs;
 *   3. a kernel writes the control block to ctrl_host, the ctrl->n walkers of
 *      dev_dst (x, v, who, key) into host, and, with hist_host, the vref and
 *      population history of the steps run (at most max_steps) to
 *      hist_host[0..) and hist_host[max_steps..);
 *   4. the call waits for the stream once.
 * dev_src and dev_dst are device walker buffers of sim->ld slots; their key
 * arrays are used when host->key is set. */
int gbdmc_sim_run_host(const gbdmc_sim_t* sim, gbdmc_host_walkers_t* host, const gbdmc_walkers_t* dev_src,
                       const gbdmc_walkers_t* dev_dst, gbdmc_ctrl_t* ctrl_dev, gbdmc_ctrl_t* ctrl_host,
                       void* scratch_dev, int64_t step_end, int32_t max_steps, double* hist_host, void* stream);

/* The two halves of a step around a potential the caller evaluates
 * (sim->pes.kind == GBDMC_PES_EXTERNAL, plain DMC): gbdmc_sim_move is
 * move_randomly (pyvibdmc.py:540-547) -- the logical walkers of src (through
 * src->idx) moved into dst in order, dst->x, who and w written; the caller
 * then writes V of the ctrl->n moved walkers to dst->v (the reference's
 * potential call, :785-793) and gbdmc_sim_branch runs birth_or_death
 * (:380-454), calc_vref (:651-661) and update_sim_arrays (:674-682) on them:
 * discrete weighting writes dst->idx (the branched population is dst
 * gathered through it), continuous weighting works in place.  The
 * branching uniforms are the injected noise->u_branch or a Philox stream
 * disjoint from the move's.  gbdmc_sim_init takes the start walkers' V from
 * w->v for this kind.  Scratch as gbdmc_sim_step. */
int gbdmc_sim_move(const gbdmc_sim_t* sim, const gbdmc_walkers_t* src, const gbdmc_walkers_t* dst,
                   gbdmc_ctrl_t* ctrl_dev, void* scratch_dev, const gbdmc_noise_t* noise, void* stream);
int gbdmc_sim_branch(const gbdmc_sim_t* sim, const gbdmc_walkers_t* dst, gbdmc_ctrl_t* ctrl_dev,
                     void* scratch_dev, const gbdmc_noise_t* noise, void* stream);

/* Batched ensemble of nrep <= GBDMC_MAX_REPLICAS independent replicas in
 * one launch per phase (persistent grid over all replicas' tiles).  sim->ld
 * is the total slot count, sim->n0 is ignored (per replica in reps), ctrl_dev
 * holds nrep control blocks and the history arrays are replica-major with
 * stride sim->hist.len.  Scratch: gbdmc_batch_scratch_bytes(reps, nrep),
 * laid out over the table's slot extent (the largest off + cap), so a call
 * may step a subset of a larger batch with a scratch sized for that subset. */
int gbdmc_batch_init(const gbdmc_sim_t* sim, const gbdmc_replica_t* reps, int32_t nrep,
                     const gbdmc_walkers_t* w, gbdmc_ctrl_t* ctrl_dev, void* scratch_dev, void* stream);
int gbdmc_batch_step(const gbdmc_sim_t* sim, const gbdmc_replica_t* reps, int32_t nrep,
                     const gbdmc_walkers_t* src, const gbdmc_walkers_t* dst, gbdmc_ctrl_t* ctrl_dev,
                     void* scratch_dev, const gbdmc_noise_t* noise, void* stream);
size_t gbdmc_batch_scratch_bytes(const gbdmc_replica_t* reps, int32_t nrep);

/* Compaction: out[off + j] = the logical walker j of `in` (through in->idx)
 * for j < ctrl[r].n of every replica; out->idx is ignored.  For the single
 * simulation pass nrep = 0 and reps = NULL (one replica over [0, sim->ld)). */
int gbdmc_walkers_compact(const gbdmc_sim_t* sim, const gbdmc_replica_t* reps, int32_t nrep,
                          const gbdmc_walkers_t* in, const gbdmc_walkers_t* out,
                          const gbdmc_ctrl_t* ctrl_dev, void* stream);

/* One step of walkers held in page-locked host memory: the reference's
 * propagate iteration (pyvibdmc.py:710-848) seen from the FFI, NumPy-style
 * walker arrays in, the branched population out.  `host` holds the compact
 * walkers [3A][sim->ld] -- x and v, plus who / f, psi, ke / w as the
 * configuration uses them, no idx -- in memory from cudaHostAlloc or
 * cudaHostRegister; the kernels read and write it directly over the host
 * link (no staging copies).  `work` is a device walker set.  The step runs
 * host -> work; with discrete weighting the branching pass then writes the
 * branched walkers (each copied c times, the np.repeat order) and the
 * control block straight into host and ctrl_host (page-locked); continuous
 * weighting compacts work -> host and copies the control block.  After the
 * stream is synchronised, host holds the ctrl_host->n walkers of the next
 * step in columns 0..n-1; after a failed step (ctrl_host->status set) it
 * still holds the walkers of before the step. */
int gbdmc_sim_step_host(const gbdmc_sim_t* sim, const gbdmc_walkers_t* host, const gbdmc_walkers_t* work,
                        gbdmc_ctrl_t* ctrl_dev, gbdmc_ctrl_t* ctrl_host, void* scratch_dev,
                        const gbdmc_noise_t* noise, void* stream);

/* Allocation-free step (no counterpart in the reference).  For callers that
 * cannot allocate device memory -- a plug-in that is handed only its input
 * and output buffers, or a host application whose own memory manager owns
 * the device and forbids other allocations -- this is gbdmc_sim_step with
 * its scratch taken from a static
 * device array of GBDMC_STATIC_SCRATCH_BYTES (1 MiB) inside the library, so
 * sim->ld is limited to gbdmc_sim_step_static_max_ld() walkers (larger ld
 * returns GBDMC_ERR_CAPACITY).  It calls no allocator.  The array is held
 * by every GPU that loads the library until the process exits.  The first
 * call on a device looks up the array's device address
 * (cudaGetSymbolAddress), so make that first call before any stream capture;
 * the address is kept for the life of the process and is not valid after a
 * cudaDeviceReset of that device.
 * All calls share the one array: calls that overlap on the GPU (other
 * streams, other threads) race and must be serialised by the caller.  The
 * scratch needs no zeroing between calls; every word a step reads is written
 * earlier in the same step. */
int gbdmc_sim_step_static(const gbdmc_sim_t* sim, const gbdmc_walkers_t* src, const gbdmc_walkers_t* dst,
                          gbdmc_ctrl_t* ctrl_dev, const gbdmc_noise_t* noise, void* stream);
size_t gbdmc_sim_step_static_max_ld(void);

/* Descendant weights: desc_dev[q] = #walkers (or sum of weights, w_dev != NULL)
 * whose ancestor id is q; desc_dev has n_parent entries and is overwritten. */
int gbdmc_desc_weights(const int32_t* who_dev, const double* w_dev, const int64_t* n_dev,
                       int64_t n_parent, double* desc_dev, void* stream);

/* np.argpartition(w, kth) (pyvibdmc.py:443-445, the walkers replaced above
 * the upper continuous-weight threshold) in the order of NumPy's portable
 * introselect, run by one 1024-thread block as inside the continuous-weight
 * step: perm_dev (n int32) receives the permutation, whose first kth entries
 * are the kth smallest weights in NumPy's order; for kth >= 3 the whole
 * permutation is NumPy's (for kth < 3 the entries from kth on may differ).
 * lpos_dev (n int32) and flags_dev (n bytes) are scratch.  0 <= kth < n.
 * perm_dev[0] = -1 reports the (unreachable below 5^16 elements) overflow of
 * the nested median-of-medians stack. */
int gbdmc_argpartition(const double* w_dev, int64_t n, int64_t kth, int32_t* perm_dev, int32_t* lpos_dev,
                       uint8_t* flags_dev, void* stream);

/* Start of a descendant-weighting window: who_dev[i] = i for i < *n_dev
 * (pyvibdmc.py:739-745, `_who_from = np.arange(len(coords))`). */
int gbdmc_desc_begin(int32_t* who_dev, const int64_t* n_dev, void* stream);

/* sizeof() of the ABI structs, for binding self-checks:
 * 0 gbdmc_sim_t, 1 gbdmc_walkers_t, 2 gbdmc_ctrl_t, 3 gbdmc_noise_t,
 * 4 gbdmc_pes_t, 5 gbdmc_trial_t, 6 gbdmc_history_t, 7 gbdmc_replica_t, 8 gbdmc_mlp_t,
 * 9 gbdmc_walkers_f32_t, 10 gbdmc_adam_param_t, 11 gbdmc_host_walkers_t; 0 for unknown ids. */
size_t gbdmc_struct_size(int32_t which);

/* ---- MLP surrogate of the water-dimer PES (BF16 tensor cores, FP32 accumulation) ----
 * Replaces the user model behind NN_Potential.getpot
 * (simulation_utilities/potential_manager.py:177-214) and the descriptor of
 * DistIt (tensorflow_descriptors/distance_descriptors.py:102-113, 154-165, 177-213):
 * the upper triangle of the Coulomb matrix z_i z_j / r_ij, normalised per
 * pair (which absorbs the charges, so the network sees (1/r - mu) / sd),
 * optionally in DistIt's sorted atom order (sort_atoms):
 * 15 descriptors -> 3 x 128 SiLU -> 1.
 * Weight matrices are bf16 and stored transposed (n-major): wNt[n*K + k]. */
#define GBDMC_MLP_HIDDEN 128
#define GBDMC_MLP_INPUT 16 /* 15 features, padded */
typedef struct {
  const uint16_t* w1t; /* [128][16]  */
  const uint16_t* w2t; /* [128][128] */
  const uint16_t* w3t; /* [128][128] */
  const float* b1;
  const float* b2;
  const float* b3;     /* [128] each */
  const float* w4;     /* [128] output weights (fp32) */
  float b4;
  float e_mean;        /* V = e_mean + e_scale * network output (hartree) */
  float e_scale;
  float hull_margin;   /* walkers with a normalised feature outside [lo-m, hi+m] use the analytic PES */
  float feat_mu[16];
  float feat_inv_sd[16];
  float feat_lo[16];
  float feat_hi[16];
  int32_t audit_every; /* walker audited (analytic PES, error recorded) with probability 1/audit_every
                          (32-bit hash h of walker, step, replica: h * audit_every < 2^32); 0 = off */
  int32_t engine;      /* 0: mma.sync BF16 kernels; 1: tcgen05 (TMEM accumulators, one thread per walker) */
  float bias_beta;     /* online bias control: c <- (1-b) c + b <V_nn - V_analytic>_audit each step, and the
                          next step's surrogate energies are V_nn - c (0 = off) */
  int32_t sort_atoms;  /* 1: descriptors in the canonical atom order of DistIt(method='coulomb',
                          sorted_atoms=[[0],[1,2],[3],[4,5]], sorted_groups=[[0,1,2],[3,4,5]])
                          (distance_descriptors.py:115-152): the hydrogens of each water by the column
                          norms of the Coulomb matrix, then the waters by their columns' summed norms;
                          0: the given order */
} gbdmc_mlp_t;

/* fp32-coordinate walkers of the surrogate path (SoA [18][ld]).  With a trial
 * wave function (sim->trial.kind = GBDMC_TRIAL_DIMER_GAUSS) the walkers also
 * carry the drift d ln psi/dx (f, [18][ld]), ln psi and the local kinetic
 * energy, all fp32, and v holds the local energy V + KE. */
typedef struct {
  float* x;
  double* v;
  int32_t* who;
  int32_t* idx;
  float* f;
  float* lnpsi;
  float* ke;
} gbdmc_walkers_f32_t;

/* Training kernels (bf16 operands, fp32 accumulation).  mma.sync m16n8k16:
 * Y[M x 128] = X[M x K] W + b (K = 16 or 128; X fp32 rounded to bf16). */
int gbdmc_mlp_gemm(const float* x_dev, int64_t m, int32_t k, const uint16_t* wt_dev, const float* bias_dev,
                   float* y_dev, void* stream);
/* G[K x 128] += X^T D over the m rows (fp32 atomics). */
int gbdmc_mlp_gemm_tn(const float* x_dev, const float* d_dev, int64_t m, int32_t k, float* g_dev, void* stream);
/* The same two GEMMs on the tcgen05 tensor cores (M = N = 128 MMAs, the accumulator in tensor memory,
 * operands staged in the canonical K-major layout; gemm_tn stages X^T and D^T and adds each CTA's partial
 * with one fp32 atomic per element). */
int gbdmc_mlp_gemm_tc(const float* x_dev, int64_t m, int32_t k, const uint16_t* wt_dev, const float* bias_dev,
                      float* y_dev, void* stream);
int gbdmc_mlp_gemm_tn_tc(const float* x_dev, const float* d_dev, int64_t m, int32_t k, float* g_dev, void* stream);
/* Two GEMMs of one weight matrix in one launch (engine 0: mma.sync, 1: tcgen05): Y0 = X0 W + b0 and
 * Y1 = X1 W + b1 (either bias may be NULL), e.g. a layer's primal and tangent streams; and
 * G += X0^T D0 + X1^T D1.  Each equals the two single calls. */
int gbdmc_mlp_gemm_pair(const float* x0_dev, const float* x1_dev, int64_t m, int32_t k, const uint16_t* wt_dev,
                        const float* bias0_dev, const float* bias1_dev, float* y0_dev, float* y1_dev, int32_t engine,
                        void* stream);
int gbdmc_mlp_gemm_tn_pair(const float* x0_dev, const float* d0_dev, const float* x1_dev, const float* d1_dev,
                           int64_t m, int32_t k, float* g_dev, int32_t engine, void* stream);
/* 1 if a bounded tensor-core wait of the tcgen05 training GEMMs gave up since the last clear (synchronises),
 * 0 if not, -1 on a CUDA error; clear != 0 resets it. */
int gbdmc_mlp_gemm_status(int32_t clear);
/* H = silu(Z), Ht = silu'(Z) Zt (Zt/Ht may be NULL). */
int gbdmc_mlp_silu_fwd(const float* z_dev, const float* zt_dev, float* h_dev, float* ht_dev, int64_t n, void* stream);
/* Zb = silu'(Z) Hb + silu''(Z) Zt Htb, Ztb = silu'(Z) Htb (Zt/Htb/Ztb may be NULL) on rows of 128 columns
 * (n a multiple of 128); with gbias_dev (may be NULL) also gbias[c] += sum over rows of Zb[., c], the
 * layer's bias gradient (fp32 atomics). */
int gbdmc_mlp_silu_bwd(const float* z_dev, const float* zt_dev, const float* hb_dev, const float* htb_dev,
                       float* zb_dev, float* ztb_dev, int64_t n, float* gbias_dev, void* stream);
/* Output layer + loss wE<(E-e)^2> + wF<(Et-et)^2>; writes dL/dH3, dL/dHt3 and accumulates dL/dw4, dL/db4,
 * loss[0] += sum (E-e)^2, loss[1] += sum (Et-et)^2.  b4 is read from b4_dev when that is not NULL. */
int gbdmc_mlp_head(const float* h3_dev, const float* ht3_dev, const float* w4_dev, float b4, const float* b4_dev,
                   const float* e_dev, const float* et_dev, int64_t m, float w_e, float w_f, float* h3b_dev,
                   float* ht3b_dev, float* gw4_dev, float* gb4_dev, double* loss_dev, void* stream);
/* The inputs of a training batch, so that a batch can be one CUDA graph: samples [off, off + b) of the data
 * set (fp64 SoA x_dev, grad_dev [18][ld], v_dev [ld]) with off = ctl_dev[1]; feat (descriptors, as
 * gbdmc_dimer_features), and along a random unit direction u of the 18 coordinates (Philox normals of
 * (seed, ctl_dev[0], sample), normalised) tang (their derivative) and et = (dV/dx . u) / e_scale; the
 * energy target e = (V - e_mean) / e_scale - *b4_dev.  ctl_dev: [0] Adam steps taken, [1] batch offset. */
int gbdmc_mlp_train_inputs(const double* x_dev, const double* v_dev, const double* grad_dev, int64_t ld, int64_t b,
                           const int64_t* ctl_dev, uint64_t seed, const float* mu_dev, const float* inv_sd_dev,
                           float e_mean, float e_scale, const float* b4_dev, int32_t sort_atoms, float* feat_dev,
                           float* tang_dev, float* et_dev, float* e_dev, void* stream);
/* One parameter of gbdmc_mlp_adam_all: fp32 values, gradient, Adam moments (n each); for a K x 128 weight
 * matrix (n = 128 K) the bf16 copies wt (transposed) and wn (row-major) to refresh, either may be NULL. */
typedef struct {
  float* p;
  float* g;
  float* m;
  float* v;
  uint16_t* wt;
  uint16_t* wn;
  int64_t n;
  int32_t k;
  int32_t pad;
} gbdmc_adam_param_t;
/* One Adam step on nq <= 8 parameters in one launch: t = ctl_dev[0] + 1, learning rate
 * lr_min + (lr0 - lr_min) (1 + cos(pi (t - 1 - t0) / steps)) / 2; every gradient is cleared after use; the
 * launch then sets ctl_dev[0] = t and advances ctl_dev[1] by batch.  ticket_dev: a device uint, zero before
 * the first call (the kernel leaves it zero). */
int gbdmc_mlp_adam_all(const gbdmc_adam_param_t* params, int32_t nq, float lr0, float lr_min, float beta1,
                       float beta2, float eps, int64_t t0, int64_t steps, int64_t batch, int64_t* ctl_dev,
                       uint32_t* ticket_dev, void* stream);
/* Adam step (t >= 1) on fp32 parameters; for a K x 128 weight matrix also refreshes its bf16 copies:
 * wt transposed (n-major, forward GEMM) and wn row-major (backward GEMM); either may be NULL. */
int gbdmc_mlp_adam(float* p_dev, const float* g_dev, float* m_dev, float* v_dev, int64_t n, float lr, float beta1,
                   float beta2, float eps, int32_t t, uint16_t* wt_dev, uint16_t* wn_dev, int32_t k, void* stream);
/* Normalised descriptors of n dimers (fp64 SoA [18][ld]); with vdir (SoA, may be NULL) also the normalised
 * directional derivative of the descriptors and et = (dV/dx . v) / e_scale from grad (SoA).  sort_atoms as in
 * gbdmc_mlp_t (the descriptors and their derivatives in the canonical atom order). */
int gbdmc_dimer_features(const double* x_dev, int64_t ld, int64_t n, const float* mu_dev, const float* inv_sd_dev,
                         const double* vdir_dev, const double* grad_dev, float e_scale, float* feat_dev,
                         float* tang_dev, float* et_dev, int32_t sort_atoms, void* stream);
/* Surrogate energies of n walkers (fp32 SoA [18][ld]); outside_dev[i] = 1 for walkers outside the training box
 * (may be NULL; not cleared).  With net->engine == 1 (tcgen05) status_dev (device int, required) is set to 1 if a
 * bounded wait for the tensor cores gave up.  n = 0 reads and writes nothing. */
int gbdmc_mlp_energy(const gbdmc_mlp_t* net, const float* x_dev, int64_t ld, int64_t n, double* v_dev,
                     int32_t* outside_dev, int32_t* status_dev, void* stream);
/* Surrogate DMC (discrete weighting, fp32 coordinates, sim->pes = the analytic dimer PES used for the audit
 * subset and the out-of-box fallback).  Step 0 energies are analytic.  audit_dev[9] (zeroed by the caller before
 * the first step): [0] audited walkers, [1] sum (V_nn - V_analytic), [2] sum (V_nn - V_analytic)^2,
 * [3] fallbacks, [4] the mixed-average bias correction c_mix (hartree: the moving average of the audited
 * errors), [5..7] bookkeeping of the bias control, [8] an offset the caller may set between steps (the
 * difference of the pure and mixed averages of the error, gbdmc_mlp_fw_*); the surrogate energies of a step
 * are V_nn - (c_mix + offset).
 * With sim->trial.kind = GBDMC_TRIAL_DIMER_GAUSS (tcgen05 engine only) the step is importance sampled
 * (pyvibdmc.py:549-612 in fp32: drift-diffusion proposal, trial at the proposal, Metropolis test, local
 * energy V_nn + KE, weights with dt_eff = dt * accepted / N).  The batch_ forms run nrep replicas laid out
 * as gbdmc_replica_t slot ranges, one control block each (scratch: gbdmc_batch_scratch_bytes); the audit
 * statistics and the bias correction are shared by all replicas. */
int gbdmc_mlp_sim_init(const gbdmc_sim_t* sim, const gbdmc_mlp_t* net, const gbdmc_walkers_f32_t* w,
                       gbdmc_ctrl_t* ctrl_dev, void* scratch_dev, void* stream);
int gbdmc_mlp_sim_step(const gbdmc_sim_t* sim, const gbdmc_mlp_t* net, const gbdmc_walkers_f32_t* src,
                       const gbdmc_walkers_f32_t* dst, gbdmc_ctrl_t* ctrl_dev, void* scratch_dev, double* audit_dev,
                       const gbdmc_noise_t* noise, void* stream);
int gbdmc_mlp_compact(const gbdmc_sim_t* sim, const gbdmc_walkers_f32_t* in, const gbdmc_walkers_f32_t* out,
                      const gbdmc_ctrl_t* ctrl_dev, void* stream);
/* Forward walking of the surrogate's error delta = V_nn - V_analytic (the descendant weights of
 * pyvibdmc.py:663-672 applied to delta): the pure-distribution average sum_s D_s delta_s / sum_s D_s over
 * a window, D_s the descendants of walker s at the window's end, against the mixed average over the same
 * walkers.  The walkers must be compact (gbdmc_mlp_batch_compact).  fw_begin: vnn_dev and outside_dev are
 * gbdmc_mlp_energy of the ld slots (outside_dev zeroed before); every live slot s gets who[s] = s and
 * delta_dev[s] = V_nn - V_analytic(fp32) (0 outside the training box).  fw_end: over the live walkers,
 * delta_dev[who].  Both write part_dev[2 * GBDMC_FW_BLOCKS]: per block (sum, count), to be summed in block
 * order.  reps/nrep as for gbdmc_mlp_batch_step. */
#define GBDMC_FW_BLOCKS 512
int gbdmc_mlp_fw_begin(const gbdmc_sim_t* sim, const gbdmc_replica_t* reps, int32_t nrep,
                       const gbdmc_walkers_f32_t* w, const gbdmc_ctrl_t* ctrl_dev, const double* vnn_dev,
                       const int32_t* outside_dev, double* delta_dev, double* part_dev, void* stream);
int gbdmc_mlp_fw_end(const gbdmc_sim_t* sim, const gbdmc_replica_t* reps, int32_t nrep,
                     const gbdmc_walkers_f32_t* w, const gbdmc_ctrl_t* ctrl_dev, const double* delta_dev,
                     double* part_dev, void* stream);
int gbdmc_mlp_batch_init(const gbdmc_sim_t* sim, const gbdmc_mlp_t* net, const gbdmc_replica_t* reps, int32_t nrep,
                         const gbdmc_walkers_f32_t* w, gbdmc_ctrl_t* ctrl_dev, void* scratch_dev, void* stream);
int gbdmc_mlp_batch_step(const gbdmc_sim_t* sim, const gbdmc_mlp_t* net, const gbdmc_replica_t* reps, int32_t nrep,
                         const gbdmc_walkers_f32_t* src, const gbdmc_walkers_f32_t* dst, gbdmc_ctrl_t* ctrl_dev,
                         void* scratch_dev, double* audit_dev, const gbdmc_noise_t* noise, void* stream);
int gbdmc_mlp_batch_compact(const gbdmc_sim_t* sim, const gbdmc_replica_t* reps, int32_t nrep,
                            const gbdmc_walkers_f32_t* in, const gbdmc_walkers_f32_t* out,
                            const gbdmc_ctrl_t* ctrl_dev, void* stream);

/* ---- measurement aids (no counterpart in the reference; used by bench.py) ----
 * gbdmc_prof_enable(1) makes every later gbdmc_sim_step record CUDA events
 * around its walker-move kernel (move + PES + weights) and its branching
 * scatter kernel, on the stream of the call; gbdmc_prof_read synchronises
 * those events, returns the summed milliseconds and launch counts, and
 * clears them.  Up to 8192 steps are recorded between reads.  Not for use
 * under stream capture. */
int gbdmc_prof_enable(int32_t on);
int gbdmc_prof_read(double* move_ms, int64_t* move_launches, double* scatter_ms, int64_t* scatter_launches);

/* Measured fp64 FMA throughput: `blocks` x 256 threads each run `iters`
 * dependent-free DFMA groups; *flops_out = flops executed.  Time it with
 * events around the call. */
int gbdmc_fp64_fma_probe(double* sink_dev, int64_t iters, int32_t blocks, double* flops_out, void* stream);

/* ---- compile-time bounds checking (no counterpart in the reference) ----
 * libgbdmc_bc.so is the same library built with -DGBDMC_BOUNDS_CHECK: every
 * data-dependent index of the step kernels (gather indices, copy positions,
 * kill-list slots, the multi-step kernel's block buffers and output) is checked
 * against its range; an index outside it sets the bit of its site (the
 * gbdmc::BoundsSite numbering: 0 plain-move gather, 1 importance-sampled
 * gather, 2 compaction gather, 3 gbdmc_sim_move gather, 4 discrete copy past
 * the capacity, 5 continuous kill-list slot or argmax, 6 multi-step block
 * buffer, 7 multi-step output, 8 surrogate copy past the capacity) and is
 * replaced by the low end of the range, so the kernel never traps.
 * gbdmc_bounds_check_enabled() is 1 in that build and 0 in libgbdmc.so;
 * gbdmc_bounds_errors(clear) synchronises the device and returns the bits set
 * since the last clear (always 0 in libgbdmc.so). */
int gbdmc_bounds_check_enabled(void);
uint32_t gbdmc_bounds_errors(int32_t clear);

#ifdef __cplusplus
}
#endif
#endif /* GBDMC_H */
