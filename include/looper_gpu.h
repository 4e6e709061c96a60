/*
 * looper_gpu.h — C ABI of the GB300 loop-cluster engine.
 *
 * This is the drop-in boundary for looper's continuous-imaginary-time loop-cluster worker
 * ("loop; path integral", path_integral.C:872-876).  Every entry point below replaces one member
 * of that worker's plug-in interface (class loop_worker : alps::parapack::mc_worker,
 * path_integral.C:57-124) or one of its parameter / observable conventions.  Plain C types only:
 * no pointer into device memory crosses this boundary; the library owns all device state.
 *
 * Errors: every function returns an int status (LG_OK = 0, negative on failure) and the message
 * of the last failure on the calling thread is available from lg_last_error().  Exceptions never
 * cross the boundary.  This replaces the worker's boost::throw_exception(std::invalid_argument /
 * logic_error / runtime_error) reporting (path_integral.C:212-213, model.h:62-80,
 * temperature.h:100, graph_impl.h:593,606, weight_impl.h:205-212).
 *
 * Threading: a handle is not thread-safe; drive each handle from one host thread.  The device
 * work of a handle is ordered on its own CUDA stream.
 */
#ifndef LOOPER_GPU_H
#define LOOPER_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------------------------- */
enum {
  LG_OK = 0,
  LG_EINVAL = -1,        /* invalid parameter (std::invalid_argument in the reference)        */
  LG_ENOMEM = -2,        /* device or host allocation failed                                  */
  LG_EDEVICE = -3,       /* CUDA error                                                         */
  LG_EUNSUPPORTED = -4,  /* model outside the supported set (e.g. sign problem, S > 1/2)      */
  LG_EITERCAP = -5,      /* a device loop hit its iteration cap and stopped                  */
  LG_EBUDGET = -6,       /* a request exceeds the memory budget                               */
  LG_ECORRUPT = -7,      /* checkpoint data rejected                                          */
  LG_ENOTREADY = -8      /* nothing to report yet                                             */
};

/* ---- lattices (ALPS LATTICE names) ---------------------------------------------------------
 * periodic, nearest neighbour: site = x + L*y + L*L*z; bond = site*dim + d joins site and
 * site + e_d.  Sublattice gauge +1/-1 by the parity of x+y+z (lattice.h:601). */
enum { LG_CHAIN = 1, LG_SQUARE = 2, LG_CUBIC = 3 };

/* ---- model / run parameters --------------------------------------------------------------
 * Replaces the alps::Parameters read by loop_worker's constructor (path_integral.C:202-305):
 * LATTICE, L (lattice_helper, lattice.h:290-315); MODEL "spin" couplings J, Jz, Jxy, h
 * (model_parameter.h:62-70, S=1/2 only); T or BETA (temperature.h:43-54); SWEEPS and
 * THERMALIZATION (montecarlo.h:41-45: THERMALIZATION defaults to SWEEPS/8);
 * DISABLE_IMPROVED_ESTIMATOR (path_integral.C:217); FORCE_SCATTER (weight_impl.h:289);
 * SEED.  NaN in jz / jxy means "not given": they then default to J (ALPS spin model). */
typedef struct lg_params {
  int lattice;                    /* LG_CHAIN, LG_SQUARE, LG_CUBIC                              */
  int L;                          /* linear size, >= 2                                          */
  double T;                       /* temperature (used when beta <= 0)                          */
  double beta;                    /* inverse temperature; > 0 overrides T                       */
  double J, Jz, Jxy;              /* couplings; H_b = Jz SzSz + Jxy/2 (S+S- + S-S+)            */
  double h;                       /* longitudinal field, H_s = -h Sz                            */
  double force_scatter;           /* FORCE_SCATTER in [0,1], default 0                          */
  uint64_t sweeps;                /* SWEEPS (measurement sweeps)                                */
  int64_t thermalization;         /* THERMALIZATION; < 0 means SWEEPS/8                         */
  uint64_t seed;                  /* SEED                                                        */
  int init_spins;                 /* 0: all up (path_integral.C:225), 1: iid from the seed      */
  int disable_improved_estimator; /* DISABLE_IMPROVED_ESTIMATOR                                  */
  int measure_correlations;       /* MEASURE[Correlations] (correlation.h:66), default 0        */
  int measure_structure_factor;   /* MEASURE[Structure Factor] (correlation.h:68), default 0    */
  int initial_site;               /* INITIAL_SITE (correlation.h:87); < 0: all pairs (default)  */
  int spin2;                      /* 2 local_S: 1 (S=1/2, default), 2 (S=1), 3 (S=3/2); S > 1/2
                                     runs on 2S virtual spin-1/2 sites per site (lattice.h
                                     virtual graph) with the random boundary matching of
                                     path_integral.C:590-613                                    */
  int algorithm;                  /* ALGORITHM: LG_PATH_INTEGRAL ("loop; path integral", default)
                                     or LG_SSE ("loop; sse": the stochastic series expansion
                                     worker of sse.C, S = 1/2 without field, run one GPU thread
                                     per chain)                                                 */
} lg_params;

enum { LG_PATH_INTEGRAL = 0, LG_SSE = 1 };

/* Fill defaults: chain, L=8, T=0.2, J=1, Jz=Jxy=NaN, h=0, SWEEPS=65536 (montecarlo.h:41),
 * THERMALIZATION=-1, SEED=29833, all spins up. */
void lg_params_default(lg_params* p);

/* Parse ALPS-style "KEY = value" lines (';' or newline separated, '#' comments) into *p.
 * Keys: LATTICE ("chain lattice" | "square lattice" | "simple cubic lattice"), L, T, BETA, J,
 * Jz, Jxy, h, FORCE_SCATTER, SWEEPS, THERMALIZATION, SEED, INITIAL_SPINS ("up" | "random"),
 * DISABLE_IMPROVED_ESTIMATOR, MEASURE[Correlations], MEASURE[Structure Factor], INITIAL_SITE,
 * local_S (1/2, 1, 3/2 ...), ALGORITHM ("loop; path integral" | "loop; sse").
 * Unknown keys are ignored, as ALPS does for keys a worker does not
 * read.  Returns LG_EINVAL with a message on a malformed value. */
int lg_params_parse(const char* text, lg_params* p);

/* ---- observables -------------------------------------------------------------------------
 * Names follow the reference's ObservableSet entries (energy.h:79-84, susceptibility.h:200-254
 * and :303-335, stiffness.h:77-78, path_integral.C:832-861) and the evaluators (energy.h:89-101,
 * susceptibility.h:340-374).  With the improved estimator (no field) the (Staggered)
 * Magnetization^2/^4 and Susceptibility entries are the improved ones; with a field they are
 * the normal estimators. */
enum {
  LG_OBS_ENERGY = 0,                 /* "Energy"                                  */
  LG_OBS_ENERGY_DENSITY,             /* "Energy Density"                          */
  LG_OBS_ENERGY2,                    /* "Energy^2"                                */
  LG_OBS_SPECIFIC_HEAT,              /* "Specific Heat" (evaluator)               */
  LG_OBS_MAGNETIZATION,              /* "Magnetization"                           */
  LG_OBS_ABS_MAGNETIZATION,          /* "|Magnetization|"                         */
  LG_OBS_MAGNETIZATION2,             /* "Magnetization^2"                         */
  LG_OBS_MAGNETIZATION4,             /* "Magnetization^4"                         */
  LG_OBS_SUSCEPTIBILITY,             /* "Susceptibility"                          */
  LG_OBS_STAG_MAGNETIZATION2,        /* "Staggered Magnetization^2"               */
  LG_OBS_STAG_MAGNETIZATION4,        /* "Staggered Magnetization^4"               */
  LG_OBS_STAG_SUSCEPTIBILITY,        /* "Staggered Susceptibility"                */
  LG_OBS_GEN_MAGNETIZATION2,         /* "Generalized Magnetization^2" (improved)  */
  LG_OBS_GEN_SUSCEPTIBILITY,         /* "Generalized Susceptibility" (improved)   */
  LG_OBS_NUM_CLUSTERS,               /* "Number of Clusters"                      */
  LG_OBS_NUM_OPERATORS,              /* operator count n_v (weight_parameter)     */
  LG_OBS_BINDER,                     /* "Binder Ratio of Magnetization"           */
  LG_OBS_STAG_BINDER,                /* "Binder Ratio of Staggered Magnetization" */
  LG_OBS_STIFFNESS,                  /* "Stiffness" (stiffness.h:116-160)        */
  LG_NUM_OBS
};

typedef struct lg_obs {
  uint64_t count;                    /* measured sweeps                                         */
  double beta, volume;               /* "Inverse Temperature", "Volume"                        */
  int improved;                      /* 1 if the improved estimator is in use                  */
  double mean[LG_NUM_OBS];
  double error[LG_NUM_OBS];          /* binning error (largest level with >= 64 bins)          */
  double tau[LG_NUM_OBS];            /* integrated autocorrelation time estimate               */
} lg_obs;

/* Observable name (the reference's ObservableSet key) for an LG_OBS_* index. */
const char* lg_obs_name(int index);

/* ---- per-sweep measurement values -----------------------------------------------------------
 * The scalar values loop_worker::run pushes into the ObservableSet after every sweep
 * (path_integral.C:832-861): its own entries (:832-836), energy::commit (energy.h:76-84),
 * susceptibility's improved or normal commit (susceptibility.h:200-254, :303-335) and
 * stiffness's (stiffness.h:124-127, :160-165), registered by init_observables
 * (path_integral.C:307-321, susceptibility.h:59-93).  A worker plug-in pushes each fetched row
 * into its ObservableSet under lg_value_name(i), so that ALPS's own binning and evaluators
 * (Specific Heat, Binder ratios) run unchanged.  Which entries a chain pushes depends on its
 * estimator and lattice (lg_value_mask); the others are NaN in a fetched row. */
enum {
  LG_VAL_TEMPERATURE = 0,               /* "Temperature"                                      */
  LG_VAL_INVERSE_TEMPERATURE,           /* "Inverse Temperature"                              */
  LG_VAL_VOLUME,                        /* "Volume"                                           */
  LG_VAL_NUMBER_OF_SITES,               /* "Number of Sites"                                  */
  LG_VAL_NUMBER_OF_CLUSTERS,            /* "Number of Clusters"                               */
  LG_VAL_ENERGY,                        /* "Energy"                                           */
  LG_VAL_ENERGY_DENSITY,                /* "Energy Density"                                   */
  LG_VAL_ENERGY2,                       /* "Energy^2"                                         */
  LG_VAL_MAGNETIZATION,                 /* "Magnetization"                                    */
  LG_VAL_MAGNETIZATION_DENSITY,         /* "Magnetization Density"                            */
  LG_VAL_ABS_MAGNETIZATION,             /* "|Magnetization|"                                  */
  LG_VAL_ABS_MAGNETIZATION_DENSITY,     /* "|Magnetization Density|"                          */
  LG_VAL_MAGNETIZATION2,                /* "Magnetization^2"                                  */
  LG_VAL_MAGNETIZATION_DENSITY2,        /* "Magnetization Density^2"                          */
  LG_VAL_MAGNETIZATION4,                /* "Magnetization^4"                                  */
  LG_VAL_MAGNETIZATION_DENSITY4,        /* "Magnetization Density^4"                          */
  LG_VAL_SUSCEPTIBILITY,                /* "Susceptibility"                                   */
  LG_VAL_GEN_MAGNETIZATION2,            /* "Generalized Magnetization^2"          (improved)  */
  LG_VAL_GEN_MAGNETIZATION_DENSITY2,    /* "Generalized Magnetization Density^2"  (improved)  */
  LG_VAL_GEN_MAGNETIZATION4,            /* "Generalized Magnetization^4"          (improved)  */
  LG_VAL_GEN_MAGNETIZATION_DENSITY4,    /* "Generalized Magnetization Density^4"  (improved)  */
  LG_VAL_GEN_SUSCEPTIBILITY,            /* "Generalized Susceptibility"           (improved)  */
  LG_VAL_STAG_MAGNETIZATION,            /* "Staggered Magnetization"              (bipartite) */
  LG_VAL_STAG_MAGNETIZATION_DENSITY,    /* "Staggered Magnetization Density"                  */
  LG_VAL_ABS_STAG_MAGNETIZATION,        /* "|Staggered Magnetization|"                        */
  LG_VAL_ABS_STAG_MAGNETIZATION_DENSITY,/* "|Staggered Magnetization Density|"                */
  LG_VAL_STAG_MAGNETIZATION2,           /* "Staggered Magnetization^2"                        */
  LG_VAL_STAG_MAGNETIZATION_DENSITY2,   /* "Staggered Magnetization Density^2"                */
  LG_VAL_STAG_MAGNETIZATION4,           /* "Staggered Magnetization^4"                        */
  LG_VAL_STAG_MAGNETIZATION_DENSITY4,   /* "Staggered Magnetization Density^4"                */
  LG_VAL_STAG_SUSCEPTIBILITY,           /* "Staggered Susceptibility"                         */
  LG_VAL_GEN_STAG_MAGNETIZATION2,       /* "Generalized Staggered Magnetization^2"            */
  LG_VAL_GEN_STAG_MAGNETIZATION_DENSITY2,/* "... Density^2"           (bipartite, improved)   */
  LG_VAL_GEN_STAG_MAGNETIZATION4,       /* "Generalized Staggered Magnetization^4"            */
  LG_VAL_GEN_STAG_MAGNETIZATION_DENSITY4,/* "... Density^4"                                   */
  LG_VAL_GEN_STAG_SUSCEPTIBILITY,       /* "Generalized Staggered Susceptibility"             */
  LG_VAL_STIFFNESS,                     /* "Stiffness"                                        */
  LG_NUM_VALUES
};

/* ObservableSet key of value i (LG_VAL_*). */
const char* lg_value_name(int index);

/* ---- one chain: the loop_worker interface ------------------------------------------------- */
typedef struct lg_chain lg_chain;

/* loop_worker::loop_worker(alps::Parameters const&)   (path_integral.C:202-305) */
int lg_create(const lg_params* p, lg_chain** out);
/* ~loop_worker   (path_integral.C:73-89) */
int lg_destroy(lg_chain* c);
/* loop_worker::run(ObservableSet&) called nsweeps times: one sweep of update + measurement each
 * (path_integral.C:323-351 -> dispatch :355-864). */
int lg_run(lg_chain* c, int64_t nsweeps);
/* loop_worker::is_thermalized() / progress()   (path_integral.C:92-93, montecarlo.h:58-61) */
int lg_is_thermalized(const lg_chain* c);
double lg_progress(const lg_chain* c);
/* ObservableSet contents after the runs so far (init_observables :307-321 + evaluators). */
int lg_observables(lg_chain* c, lg_obs* out);
/* loop_worker::save / load (path_integral.C:111-124): mcs, spins, operator string.
 * lg_save with buf == NULL stores the required size in *size.  lg_load rejects a blob whose
 * checksum, version, lattice, size or operators do not check (LG_ECORRUPT) and a configuration
 * that is not periodic in imaginary time (LG_EINVAL, as lg_set_state); the chain then keeps its
 * state. */
int lg_save(lg_chain* c, void* buf, size_t* size);
int lg_load(lg_chain* c, const void* buf, size_t size);
/* Exchange Monte Carlo hooks (path_integral.C:97-109). */
int lg_set_beta(lg_chain* c, double beta);

/* Per-sweep values (LG_VAL_*): the ObservableSet pushes of loop_worker::run, one row of
 * LG_NUM_VALUES doubles per measurement sweep (sweeps after THERMALIZATION, the ones
 * lg_observables accumulates).  lg_keep_values(c, 1) starts keeping the rows of the sweeps that
 * follow (off by default); lg_fetch_values moves up to cap rows, oldest first, into out
 * (cap * LG_NUM_VALUES doubles) and stores the number of rows in *n.  *mask receives bit i set
 * for every value the chain pushes: the Generalized entries only with the improved estimator
 * (no field, path_integral.C:217), the Staggered ones only on a bipartite lattice
 * (susceptibility.h:75-93).  Works for members of a batch too (lg_batch_chain). */
int lg_value_mask(const lg_chain* c, uint64_t* mask);
int lg_keep_values(lg_chain* c, int on);
int lg_fetch_values(lg_chain* c, double* out, int64_t cap, int64_t* n);

/* ---- spin correlations and structure factor (correlation.h:38-300) ------------------------
 * The reference's normal estimator of looper::correlation, measured from the tau = 0 spins at
 * the end of every measurement sweep (normal_estimator::collector::commit, correlation.h:
 * 222-296).  A chain measures them when created with measure_correlations or
 * measure_structure_factor.  Entry i of the N-entry vectors:
 *   LG_CORR_SPIN       "Spin Correlations": the displacement with site index i, i.e.
 *                      (x, y, z) = (i % L, (i / L) % L, i / L^2), averaged over all pairs
 *                      (correlation.h:248-264, multiplicity 1/N); with INITIAL_SITE o, the pair
 *                      (o, site i) (:236-247).  Value 1/4 <(1 - 2 s_a)(1 - 2 s_b)>.
 *   LG_CORR_STAGGERED  "Staggered Spin Correlations": the same times the gauges of both sites.
 *   LG_SFAC            "Spin Structure Factor" (:268-281): momentum k = 2 pi (x, y, z) / L with
 *                      each component taken into (-pi, pi]; the Fourier transform of the
 *                      all-pairs correlations (needs measure_structure_factor).
 * mean and err (err may be NULL) receive N doubles; err is the binning error over the bins of
 * up to 64 sweeps (the record chunks).  LG_EINVAL if the chain does not measure that kind. */
enum { LG_CORR_SPIN = 0, LG_CORR_STAGGERED = 1, LG_SFAC = 2 };
int lg_correlations(lg_chain* c, int kind, double* mean, double* err);
/* Test seam: the exact integer sums behind the correlations.  which = 0: sums[r] over the
 * measured sweeps of sum_i m_i m_{i+r} (all pairs, m = 1 - 2 s); which = 1: of m_o m_r (with
 * INITIAL_SITE o).  N entries; *nsweeps receives the number of measured sweeps. */
int lg_correlation_sums(lg_chain* c, int which, int64_t* sums, int64_t* nsweeps);
double lg_weight_parameter(lg_chain* c);
double lg_log_weight(double gw, double beta);
/* Message of the last failure on this thread. */
int lg_last_error(char* buf, size_t n);

/* ---- test seams --------------------------------------------------------------------------
 * Persistent configuration: spins at tau = 0 (0 up, 1 down) and the off-diagonal operators
 * (bond, FP64 time in [0,1)), time ordered.  *n receives the operator count.  lg_set_state
 * returns LG_EINVAL for an operator out of range and, at S = 1/2, for a site with an odd number
 * of operators (its world line would not be periodic in imaginary time). */
int lg_get_state(lg_chain* c, int32_t* spins, int32_t* bonds, double* times, int64_t cap,
                 int64_t* n);
int lg_set_state(lg_chain* c, const int32_t* spins, const int32_t* bonds, const double* times,
                 int64_t n, uint64_t sweep);
/* Raw per-sweep measurement records (LG_RECORD_WORDS uint64 each, exact integer sums) of every
 * sweep run so far whose records have not been fetched, oldest first. */
#define LG_RECORD_WORDS 32
int lg_fetch_records(lg_chain* c, uint64_t* out, int64_t cap, int64_t* n);
/* Keep raw records for lg_fetch_records (off by default). */
int lg_keep_records(lg_chain* c, int on);
/* Test seam (no counterpart in the reference): the union-find retry cap per union.  0 restores
 * the default (2^22); a negative value lets no union run, so that the next sweep stops with
 * LG_EITERCAP.  After LG_EITERCAP the arena's state is lost and every lg_run reports the error
 * again, until lg_load / lg_set_state restores a single chain's state. */
int lg_set_iteration_cap(lg_chain* c, int cap);
/* Test seam (no counterpart in the reference): n sweeps run kernel by kernel, with structural
 * checks after insertion, merge, cluster sums and the end of each sweep (vertex ranges inside
 * their regions and time ordered, segment offsets and vertex <-> segment links consistent,
 * union-find pointers decreasing and compressed, off-diagonal lists ordered and of even length
 * per spin-1/2 site).  Every index is range-checked before use.  The sweeps count as done and
 * give the same trajectory as lg_run.  LG_EDEVICE names the first failed check. */
int lg_validate_sweeps(lg_chain* c, int64_t n);

/* Cluster labels of a given cluster-construction configuration, computed on the GPU by the
 * segment union-find.  The configuration is a time-ordered vertex list (bond, graph 0..3) on a
 * periodic lattice.  Labels follow the reference's fragment numbering and id assignment
 * (graph_impl.h:285-288, path_integral.C:482, union_find.h:324-343 with the deterministic
 * unify of union_find.h:231-233): fragment i < N is the bottom of site i, fragment N + k the
 * k-th graph-0 vertex in time order; ids increase with the smallest fragment index of a cluster.
 * labels must hold N + (number of graph-0 vertices) entries. */
int lg_uf_label(int lattice, int L, int64_t nops, const int32_t* bonds, const int32_t* graphs,
                int32_t* labels, int64_t cap, int64_t* nfrag, int64_t* nc);

/* Allocation-free variant of lg_uf_label, for callers that cannot call cudaMalloc: a plug-in
 * whose host framework owns every device allocation through its own pool, or a latency-critical
 * path that cannot take the device-wide synchronisation of cudaFree.
 * This entry point has no counterpart in the reference.
 * d_bonds, d_graphs (nops entries) and d_labels (N + number of graph-0 vertices entries) are
 * device pointers owned by the caller; stream is a cudaStream_t (NULL: the default stream).
 * All intermediate data live in a fixed 32 MiB static device array that each GPU loading this
 * library holds until the process exits.  Limits: 16384 sites and 262144 vertices; larger inputs
 * return LG_EBUDGET.  The first call on a device looks up that array's address (make it before
 * any stream capture); the address is kept for the life of the process, so do not call this
 * entry point on a device after cudaDeviceReset.  Calls share the array: calls whose device work
 * overlaps race and must be serialised.  The call synchronises its stream once, to return
 * *nfrag and *nc. */
int lg_uf_label_static(int lattice, int L, int64_t nops, const int32_t* d_bonds,
                       const int32_t* d_graphs, int32_t* d_labels, int64_t* nfrag, int64_t* nc,
                       void* stream);

/* ---- batched chains: many independent chains in one ragged arena -------------------------- */
typedef struct lg_batch lg_batch;
int lg_batch_create(int n, const lg_params* p, lg_batch** out);
int lg_batch_destroy(lg_batch* b);
/* nsweeps sweeps of every chain (each chain stops at THERMALIZATION + SWEEPS). */
int lg_batch_run(lg_batch* b, int64_t nsweeps);
int lg_batch_observables(lg_batch* b, int chain, lg_obs* out);
int lg_batch_size(const lg_batch* b);
/* Total sites and sweeps done so far (for throughput accounting). */
int lg_batch_stats(const lg_batch* b, int64_t* total_sites, int64_t* site_sweeps);
/* Access one chain of a batch through the single-chain test seams. */
lg_chain* lg_batch_chain(lg_batch* b, int i);
/* lg_validate_sweeps for a whole arena (test seam). */
int lg_batch_validate_sweeps(lg_batch* b, int64_t n);

/* ---- launch shapes and the autotuner (no counterpart in the reference) ---------------------
 * The shape of an arena's sweep launches.  No shape changes any result (trajectories, records
 * and observables are bit-identical under every shape); it only changes speed.
 *   insert_k     chains whose expected endpoints per site, 2 beta W N_bonds / N, are below this
 *                insert operators with a thread per bond, the others with a warp per site
 *                (0: all warp, a huge value: all thread)
 *   narrow_k     the same split for the per-site merge and list compaction
 *   acc_tile     segments per CTA of the cluster-sum accumulation: 512, 1024 or 2048
 *   cl_tile      segments per CTA of the cluster flip / estimator kernel: 2048, 4096 or 8192
 *   union_warps  warps per CTA of the union-find kernel of union_mode 0 and 1: 4, 8 or 16
 *   resident     1: the chain-resident path, where every chain of the arena qualifies (S = 1/2,
 *                no correlation measurement, a sweep's operators within one CTA's shared memory):
 *                one CTA per chain runs a whole chunk of up to 64 sweeps in one launch, with the
 *                sweep's vertices, segments and union-find forest in shared memory; 0: the grid
 *                path (one CUDA graph of grid-wide kernels per sweep).  lg_create and
 *                lg_batch_create start small arenas on the resident path; a chain that outgrows a
 *                CTA moves to the grid path by itself.
 *   union_mode   how the union-find runs: 0, every union in one lock-free pass with a lane per
 *                vertex; 1, in arenas of spin-1/2 chains the lower-leg unions of the non-crossing
 *                vertices (a matching of segments that are all still roots) first, one plain
 *                store each, then the rest as in 0; 2 (default), those pairs first where 1 allows
 *                them, then the rest with each warp's unions balanced over its lanes. */
typedef struct lg_shape {
  double insert_k;
  double narrow_k;
  int acc_tile;
  int cl_tile;
  int union_warps;
  int resident;
  int union_mode;
} lg_shape;

/* Autotuner: times trial_sweeps sweeps per candidate shape (device events, flush_bytes of L2
 * flush before each sweep) and keeps the fastest shape, searching the merge split, then the
 * insertion split, then each tile size; a candidate replaces the kept shape only when it is at
 * least 2% faster.  The timed sweeps are the chains' own sweeps and count as done.
 * chosen (may be NULL) receives the shape kept; report (may be NULL) a line per candidate. */
int lg_batch_autotune(lg_batch* b, int trial_sweeps, size_t flush_bytes, lg_shape* chosen,
                      char* report, size_t report_len);
/* The same for a single chain created with lg_create. */
int lg_autotune(lg_chain* c, int trial_sweeps, size_t flush_bytes, lg_shape* chosen, char* report,
                size_t report_len);
int lg_batch_get_shape(const lg_batch* b, lg_shape* out);
/* Fix the shape by hand (LG_EINVAL for values outside the lists above). */
int lg_batch_set_shape(lg_batch* b, const lg_shape* in);
/* The same for a single chain created with lg_create. */
int lg_get_shape(const lg_chain* c, lg_shape* out);
int lg_set_shape(lg_chain* c, const lg_shape* in);

/* ---- exchange Monte Carlo (parallel tempering) over a temperature ladder ------------------
 * Replaces ALPS parapack's exchange worker around loop_worker (path_integral.C:874-875), with
 * the worker's hooks weight_parameter() = operator count n and log_weight(n, beta) = n log beta
 * (path_integral.C:98-109).  Temperature t of the ladder betas[0..n) runs as one chain of a
 * single arena (SEED of chain i: lg_exchange_chain_seed(SEED, i)).  Every `interval` sweeps the
 * neighbouring temperatures (t, t+1), t even and t odd in alternate steps, try to swap with
 * probability min(1, exp((n_i - n_j)(log beta_{t+1} - log beta_t))); a swap exchanges the two
 * chains' inverse temperatures.  Observables are accumulated per temperature. */
typedef struct lg_exchange lg_exchange;
uint64_t lg_exchange_chain_seed(uint64_t seed, int i);
int lg_exchange_create(const lg_params* p, int nbeta, const double* betas, lg_exchange** out);
int lg_exchange_destroy(lg_exchange* x);
/* nsweeps sweeps of every temperature, with an exchange step every `interval` sweeps (counted
 * across calls). */
int lg_exchange_run(lg_exchange* x, int64_t nsweeps, int interval);
/* Observables at temperature index t (the sweeps measured there, whichever chain held it). */
int lg_exchange_observables(lg_exchange* x, int t, lg_obs* out);
/* chain_of_temp[nbeta]; attempts / accepts[nbeta - 1] per neighbouring pair (any may be NULL). */
int lg_exchange_state(const lg_exchange* x, int32_t* chain_of_temp, uint64_t* attempts,
                      uint64_t* accepts);
/* Chain c of the ladder through the single-chain test seams (its state, records). */
lg_chain* lg_exchange_chain(lg_exchange* x, int c);

/* ---- request server: continuous batching over one device arena ---------------------------
 * Serving form of the worker (no counterpart in the reference, whose scheduler runs one
 * worker per clone; see path_integral.C:872-876 for the worker it batches).  Requests (lg_params)
 * are queued, admitted in arrival order while their estimated device memory (from the expected
 * operator count beta * W * N_bonds) fits the budget, and run together in one arena whose sweeps
 * are CUDA graphs; chain state stays on the device between sweeps and moves device to device when
 * the arena is rebuilt.  Each result equals the result of the same request run alone (lg_create
 * + lg_run + lg_observables), bit for bit. */
typedef struct lg_server lg_server;
typedef struct lg_server_config {
  double budget_bytes;       /* device memory budget for admitted requests (default 150e9)    */
  int sweeps_per_tick;       /* sweeps between admission / retirement points (default 16)    */
  double rebuild_interval_s; /* minimum time between arena rebuilds while busy (0.02 s)      */
  int max_active;            /* maximum chains in one lane's arena (default 4096)            */
  int lanes;                 /* size classes, each with its own arena, host thread and CUDA
                                stream, run side by side (1..4, default 2): a request goes to
                                the lane of its expected operators per sweep                   */
} lg_server_config;
typedef struct lg_result {
  uint64_t id;
  int status;                /* LG_OK, or LG_EBUDGET when the request can never fit          */
  double t_submit, t_start, t_finish;   /* seconds since lg_server_create                    */
  uint64_t sweeps;           /* THERMALIZATION + SWEEPS run                                  */
  int64_t sites;
  lg_obs obs;
} lg_result;
typedef struct lg_server_stats {
  uint64_t submitted, completed, rejected, rebuilds;
  int64_t site_sweeps;       /* sweeps x sites of active chains run so far                   */
  int64_t queued;
  double active_bytes;
  double elapsed_s;
} lg_server_stats;
void lg_server_config_default(lg_server_config* c);
/* Estimated device bytes of one request (the admission figure); < 0 for invalid parameters. */
double lg_request_bytes(const lg_params* p);
int lg_server_create(const lg_server_config* c, lg_server** out);
int lg_server_submit(lg_server* s, const lg_params* p, uint64_t* id);
/* Completed results since the last poll (non-blocking). */
int lg_server_poll(lg_server* s, lg_result* out, int cap, int* n);
/* Block until every submitted request finished (LG_ENOTREADY on timeout). */
int lg_server_wait(lg_server* s, double timeout_s);
int lg_server_get_stats(lg_server* s, lg_server_stats* out);
int lg_server_destroy(lg_server* s);

/* ---- measurement seams (benchmarks) -------------------------------------------------------
 * Run n sweeps of every chain of a handle (as lg_run / lg_batch_run), each sweep bracketed by
 * CUDA events on the engine's own stream, with a device write of flush_bytes (an L2 flush)
 * between sweeps outside the brackets.  ms[i] receives the device time of sweep i. */
int lg_time_sweeps(lg_chain* c, int64_t n, size_t flush_bytes, float* ms);
int lg_batch_time_sweeps(lg_batch* b, int64_t n, size_t flush_bytes, float* ms);
/* Per-kernel profile: n sweeps launched kernel by kernel with an event after every launch;
 * kernel_ms[k] accumulates the device time of kernel k (lg_num_kernels() entries), *vertices
 * the operators processed (summed over sweeps and chains). */
int lg_profile_sweeps(lg_chain* c, int64_t n, size_t flush_bytes, double* kernel_ms,
                      int64_t* vertices);
int lg_batch_profile_sweeps(lg_batch* b, int64_t n, size_t flush_bytes, double* kernel_ms,
                            int64_t* vertices);
int lg_num_kernels(void);
const char* lg_kernel_name(int k);

/* ---- build / device info ------------------------------------------------------------------ */
/* Number of device kernel launches issued by this process so far (all handles). */
uint64_t lg_kernel_launches(void);
/* Bytes this library has copied host -> device and device -> host so far (all handles); either
 * pointer may be NULL.  A measurement seam: the end-to-end benchmark counts its transfers. */
void lg_copy_bytes(uint64_t* h2d, uint64_t* d2h);
/* Version string (engine and CUDA). */
const char* lg_version(void);

#ifdef __cplusplus
}
#endif

#endif /* LOOPER_GPU_H */
