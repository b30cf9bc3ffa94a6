/*
 * tdda.h -- C ABI of the GB300-native DDA solve path (libtdda.so).
 *
 * The library replaces the FFT-accelerated interaction product and the
 * BiCGSTAB solve of Topo-DDA (AProductCore / DDAModel).  Every entry point
 * below names the reference interface it stands in for.  Plain C types only:
 * complex vectors are interleaved doubles (re, im) -- the storage of
 * std::complex<double> and Eigen::VectorXcd -- and dipole vectors are AoS
 * [x, y, z] per dipole in the order of R, as in the reference.
 *
 * Conventions
 *   - every function returns a tdda_status; nothing throws across the ABI;
 *   - calls are synchronous (the result is ready when the call returns), like
 *     the reference; each core owns one CUDA stream;
 *   - handles are not thread-safe; models that share a core must not be used
 *     from two threads at once (the reference shares one core's scratch
 *     between models the same way, EvoDDAModel.h:14);
 *   - `mem` says whether a vector argument is host or device memory.
 */
#ifndef TDDA_H_
#define TDDA_H_

#ifdef __cplusplus
extern "C" {
#endif

#define TDDA_ABI_VERSION 1

typedef enum tdda_status {
    TDDA_OK = 0,
    TDDA_ERR_INVALID_ARGUMENT = 1,
    TDDA_ERR_CUDA = 2,
    TDDA_ERR_OUT_OF_MEMORY = 3,
    TDDA_ERR_UNSUPPORTED = 4,
    TDDA_NOT_CONVERGED = 5, /* iteration limit reached (DDAModel.cpp:256-259) */
    TDDA_BREAKDOWN = 6,     /* r0.rl == 0 stop (DDAModel.cpp:193-216) */
    TDDA_ERR_NAN = 7,       /* a BiCGSTAB scalar became NaN or infinite */
    TDDA_ERR_NO_DEVICE = 8
} tdda_status;

typedef enum tdda_method { TDDA_METHOD_LDR = 0, TDDA_METHOD_FCD = 1 } tdda_method;
typedef enum tdda_memory { TDDA_MEM_HOST = 0, TDDA_MEM_DEVICE = 1 } tdda_memory;
typedef enum tdda_precision {
    TDDA_FP64 = 0,       /* complex128 FFT convolution and Krylov vectors */
    TDDA_FP32_REFINE = 1, /* complex64 FFT and Krylov vectors, double-float dot sums, and an
                            outer residual of the FP64 vectors (double-float product, ~44 bits,
                            on the compiled grids; FP64 product elsewhere) with iterative
                            refinement */
    TDDA_FP32_JACOBI = 2  /* TDDA_FP32_REFINE whose inner BiCGSTAB is right-preconditioned by
                            the diagonal al (Jacobi): it solves (A D^-1) y = r with D = diag(al)
                            and corrects P by D^-1 y.  The outer FP64 residual check is the same,
                            so results meet the same tolerance; the inner iterates differ from
                            the reference's recurrence.  No counterpart in the reference.  For
                            the solves (tdda_solve_batch, tdda_solve_multi_precision, the server),
                            not for single products */,
    TDDA_FP32_AUTO = 3    /* per right-hand side, TDDA_FP32_JACOBI where its |al| varies by more
                            than 4x over the dipoles (densities that mix near-vacuum and dense
                            dipoles), else TDDA_FP32_REFINE; one small reduction per solve.  No
                            counterpart in the reference */
} tdda_precision;
typedef enum tdda_field {
    TDDA_FIELD_P = 0,
    TDDA_FIELD_E = 1,
    TDDA_FIELD_AL = 2,
    TDDA_FIELD_DIEL = 3,
    TDDA_FIELD_EINTERNAL = 4
} tdda_field;

typedef struct tdda_core_desc {
    int Nx, Ny, Nz;          /* lattice box (CoreStructure get_Nx/Ny/Nz) */
    int N;                   /* number of dipoles */
    const int* R;            /* 3N lattice indices, host memory (CoreStructure get_R) */
    double d;                /* lattice spacing */
    double lam;              /* vacuum wavelength */
    double nback;            /* background refractive index */
    const double* material;  /* nmat complex permittivities (re, im), host memory */
    int nmat;
    int method;              /* TDDA_METHOD_LDR or TDDA_METHOD_FCD */
    int max_rhs;             /* right-hand sides a batched solve may carry (>= 1) */
    int device;              /* CUDA device ordinal */
} tdda_core_desc;

typedef struct tdda_solve_info {
    int status;            /* tdda_status of this right-hand side */
    int iterations;        /* ITERATION as DDAModel::get_ITERATION reports it */
    double error;          /* |r| / |E| of the recursive residual at the end */
    double true_residual;  /* |E - A P| / |E| recomputed in FP64 (mixed precision only, else -1) */
    int outer_iterations;  /* refinement steps (mixed precision only, else 0) */
    int inner_iterations;  /* FP32 BiCGSTAB iterations summed over refinement steps */
} tdda_solve_info;

typedef struct tdda_core_s tdda_core;
typedef struct tdda_model_s tdda_model;

/* library ------------------------------------------------------------- */
int tdda_abi_version(void);
/* message of the last error on this thread ("" if none) */
const char* tdda_last_error(void);
/* number of visible CUDA devices (0 without a GPU; never fails) */
int tdda_device_count(void);

/* core: one lattice at one wavelength ---------------------------------- */
/* Replaces AProductCore::AProductCore(CStr, lam, material, nback, method)
 * (AProductCore.h:51, AProductCore.cpp:12-249): material normalisation,
 * Green tensor on the padded grid, its spectrum -- all on the device. */
tdda_status tdda_core_create(const tdda_core_desc* desc, tdda_core** out);
/* AProductCore's periodic constructor (AProductCore.cpp:251-536): the lattice
 * repeats with period Lm along x and Ln along y (nm).  The interaction tensor
 * at each offset is the sum of its images m in [-MAXm, MAXm], n in [-MAXn,
 * MAXn], each damped by exp(-(0.01 K r)^4) (AProductCore.cpp:573-586).  The
 * material bump of this constructor applies below |eps| = 1.01 (:263-268).
 * Everything after construction is as tdda_core_create. */
tdda_status tdda_core_create_periodic(const tdda_core_desc* desc, int MAXm, int MAXn, double Lm, double Ln,
                                      tdda_core** out);
/* Replaces AProductCore::~AProductCore (AProductCore.cpp:538-558). */
tdda_status tdda_core_destroy(tdda_core* core);
/* AProductCore::get_K / get_material (AProductCore.h:72,75) and the FFT grid
 * chosen per axis.  Any output pointer may be NULL. */
tdda_status tdda_core_info(const tdda_core* core, double* K, int* grid3, double* material_norm);
/* y = A_offdiag b, 3N complex (AProductCore::Aproduct, AProductCore.h:56,
 * AProductCore.cpp:697-758).  precision TDDA_FP32_REFINE runs the complex64
 * convolution once (no refinement) for error studies. */
tdda_status tdda_aproduct(tdda_core* core, int precision, const double* b, double* y, int mem);
/* The LDR interaction tensor at the offset (x, y, z) nm
 * (AProductCore::LDR_inter, AProductCore.h:80): out12 = xx, xy, xz, yy, yz,
 * zz as (re, im).  Host arithmetic, as in the reference. */
tdda_status tdda_core_ldr_inter(const tdda_core* core, double x, double y, double z, double* out12);
/* AProductCore::A_dic_generator(x, y, z) (AProductCore.cpp:560-571): the
 * core's interaction tensor at the offset (x, y, z) nm, LDR or FCD
 * (AProductCore.cpp:625-695, Si/Ci interpolated as SiCi.cpp:27-47 in tables
 * of Si(0.1 k), Ci(0.1 k), k = 1 .. 999999); same output layout as
 * tdda_core_ldr_inter. */
tdda_status tdda_core_interaction(const tdda_core* core, double x, double y, double z, double* out12);

/* model: incident field, polarisability and solve state ----------------- */
/* Replaces DDAModel::DDAModel(Core, n_K, E0, n_E0) (DDAModel.h:34,
 * DDAModel.cpp:12-69).  diel_old: the core structure's 3N densities
 * (CoreStructure get_diel_old), host memory. */
tdda_status tdda_model_create(tdda_core* core, const double* nK, double E0, const double* nE0,
                              const double* diel_old, tdda_model** out);
tdda_status tdda_model_destroy(tdda_model* model);
/* DDAModel::UpdateAlpha (DDAModel.cpp:470-487) for new 3N densities. */
tdda_status tdda_model_update_alpha(tdda_model* model, const double* diel_old);
/* DDAModel::UpdateAlphaSingle (DDAModel.cpp:489-528) after the density of
 * dipole idx became `value` (CoreStructure::UpdateStrSingle). */
tdda_status tdda_model_update_alpha_single(tdda_model* model, int idx, double value);
/* DDAModel::change_E / reset_E / InitializeP (DDAModel.cpp:453-468, 731-733).
 * InitializeP with P = NULL sets P = 0 on the device without a transfer. */
tdda_status tdda_model_change_E(tdda_model* model, const double* E, int mem);
tdda_status tdda_model_reset_E(tdda_model* model);
tdda_status tdda_model_initialize_P(tdda_model* model, const double* P, int mem);
/* y = A b + al b (DDAModel::Aproductwithalb, DDAModel.cpp:577-586). */
tdda_status tdda_model_aproduct_with_alb(tdda_model* model, const double* b, double* y, int mem);
/* DDAModel::bicgstab(MAX_ITERATION, MAX_ERROR) (DDAModel.cpp:131-260), FP64.
 * info may be NULL. */
tdda_status tdda_model_bicgstab(tdda_model* model, int max_it, double max_err, tdda_solve_info* info);
/* The same solve in mixed precision with FP64 refinement to max_err. */
tdda_status tdda_model_solve_mixed(tdda_model* model, int max_it, double max_err, tdda_solve_info* info);
/* DDAModel::update_E_in_structure (DDAModel.cpp:567-575). */
tdda_status tdda_model_update_E_in_structure(tdda_model* model);
/* DDAModel::get_P / get_Einternal / get_al (DDAModel.h:50-56) and E, diel:
 * copies 3N complex into out. */
tdda_status tdda_model_get(const tdda_model* model, int field, double* out, int mem);
/* DDAModel::get_ITERATION (DDAModel.h:59). */
int tdda_model_iterations(const tdda_model* model);

/* The field at off-lattice points from the model's current P:
 * E(r) = E0 nE0 exp(i K nK.r) - sum_i A(r - d R_i) P_i, with A the LDR tensor
 * (ObjPointEDDAModel, ObjDDAModel.cpp:20-96; DDAModel::solve_E,
 * DDAModel.cpp:530-565, which takes lattice indices: pass d * RResult).
 * points: 3*npts doubles in nm; E: 3*npts complex (interleaved doubles);
 * both in host or device memory per mem.  FP64; a point on a dipole site
 * takes the zero tensor for that dipole. */
tdda_status tdda_model_field_at(tdda_model* model, int npts, const double* points, double* E, int mem);

/* Adjoint sensitivity of the design densities, the product of the adjoint
 * field with the derivative of the system matrix (EvoDDAModel.cpp:610-638):
 *   s[i] = sum over the dipoles j of parameter i of
 *          Re( sum_c lambda[3j+c] * dal_j/drho_j * P[3j+c] )
 * with P the forward model's polarisation, lambda = sum_k coef[k] P(adj[k])
 * (the adjoint solutions, 1 <= nadj <= 8, coef as nadj interleaved complex),
 * and dal/drho the derivative of the forward model's inverse LDR
 * polarisability (tools.cpp:617-630) through its density interpolation
 * (DDAModel.cpp:54-63; 0 above density 1, where the table is piecewise
 * constant).  Parameter i owns dipoles[offsets[i] .. offsets[i+1]-1] (the
 * reference's Paratogeometry lists).  FP64, each sum in list order.  The
 * reference's gradient is devx - s (EvoDDAModel.cpp:640); for a point-|E|^2
 * objective with coef = conj(E_obs) over the basis adjoints it is -2 s. */
tdda_status tdda_model_density_gradient(const tdda_model* fwd, int nadj, tdda_model* const* adj, const double* coef,
                                        int nparam, const int* offsets, const int* dipoles, double* s);
/* batched solve: n models on one core, one launch per pass -------------- */
/* The forward and adjoint solves of EvoDDAModel::EvoOptimization
 * (EvoDDAModel.cpp:435-436, 596-600), or several incidences on one lattice,
 * solved together.  n <= max_rhs of the core.  infos may be NULL. */
tdda_status tdda_solve_batch(tdda_model* const* models, int n, int precision, int max_it, double max_err,
                             tdda_solve_info* infos);

/* cross-lattice batched solve: FP32+refine solves of n models whose cores
 * hold different lattices (box, dipoles, spacing, wavelength, material) on one
 * FFT grid shape (tdda_core_info's grid3) and one device.  The FP32 inner
 * solves of all n run in one launch per pass kernel (each right-hand side reads
 * its own lattice, cellmap and Green spectrum); each refinement residual runs
 * on its model's own core.  The reference solves one structure at a time with
 * one shared core (main.cpp:577-598); here each result is bit-identical to the
 * model's tdda_model_solve_mixed alone.  1 <= n <= 64; infos may be NULL. */
tdda_status tdda_solve_multi(tdda_model* const* models, int n, int max_it, double max_err,
                             tdda_solve_info* infos);
/* tdda_solve_multi with the inner solves' precision: TDDA_FP32_REFINE (the same
 * as tdda_solve_multi), TDDA_FP32_JACOBI or TDDA_FP32_AUTO. */
tdda_status tdda_solve_multi_precision(tdda_model* const* models, int n, int precision, int max_it,
                                       double max_err, tdda_solve_info* infos);

/* serving loop: continuous batching of solve requests ------------------- */
/* Requests queue in arrival order; workers run concurrently on their own CUDA
 * streams.  Operators (lattice, spacing, wavelength, material, nback: the core
 * and its Green spectrum) stay resident after their requests, with a pool of
 * their models, and later requests of the same operator reuse them; idle ones
 * are evicted least recently used first when admission needs the memory.
 * FP32+refine: a worker runs a session of max_group slots for lattices of one
 * FFT grid shape (tdda_solve_multi's batching) and, between rounds of at most
 * 32 inner steps, frees finished slots and admits queued requests of that
 * shape (continuous batching).  FP64: a worker solves the first request that
 * fits with the queued requests of its operator in one batched solve.
 * Admission is first fit under the HBM budget.  No counterpart in the
 * reference, which solves one structure at a time (main.cpp:577-598); each
 * result equals the same request solved alone. */
typedef enum tdda_request_state {
    TDDA_REQ_QUEUED = 0,
    TDDA_REQ_RUNNING = 1,
    TDDA_REQ_DONE = 2,
    TDDA_REQ_FAILED = 3
} tdda_request_state;

typedef struct tdda_server_desc {
    int device;
    double hbm_budget_bytes;  /* device memory the requests in flight may hold */
    int workers;              /* requests solved concurrently (one stream each) */
    int precision;            /* TDDA_FP64, TDDA_FP32_REFINE, TDDA_FP32_JACOBI or TDDA_FP32_AUTO */
    int max_it;
    double tol;
    int max_group;            /* right-hand sides of one batched solve, or the slots of one
                                 FP32+refine session (<= 64) */
    int dry_run;              /* scheduler only: no device work, a request takes dry_run_ms */
    double dry_run_ms;
} tdda_server_desc;

typedef struct tdda_request_desc {
    int Nx, Ny, Nz, N;
    const int* R;             /* 3N lattice indices */
    double d, lam, nback;
    const double* material;   /* nmat complex */
    int nmat;
    const double* diel_old;   /* 3N densities */
    int nrhs;                 /* incidences solved on this structure */
    const double* nK;         /* 3 x nrhs */
    const double* nE0;        /* 3 x nrhs */
    const double* E0;         /* nrhs */
} tdda_request_desc;

typedef struct tdda_request_info {
    int state;                /* tdda_request_state */
    int status;               /* worst tdda_status over the right-hand sides */
    double t_submit, t_start, t_done;  /* seconds on the server clock */
    int iterations;           /* largest iteration count over the right-hand sides */
    double error;             /* largest final relative residual */
    double bytes;             /* device bytes admitted for the request */
    int group;                /* right-hand sides sharing its launches when it was admitted */
} tdda_request_info;

typedef struct tdda_server_s tdda_server;

tdda_status tdda_server_create(const tdda_server_desc* desc, tdda_server** out);
/* copies the request; *id identifies it */
tdda_status tdda_server_submit(tdda_server* server, const tdda_request_desc* req, unsigned long long* id);
/* state and timings of a request; wait != 0 blocks until it has finished.  P,
 * if not NULL, receives the 3N x nrhs complex polarisations (host memory). */
tdda_status tdda_server_result(tdda_server* server, unsigned long long id, int wait, tdda_request_info* info,
                               double* P);
/* queued and running requests, device bytes in flight now and at most */
tdda_status tdda_server_stats(tdda_server* server, int* queued, int* running, double* bytes, double* peak_bytes);
/* seconds since the server was created */
double tdda_server_clock(const tdda_server* server);
/* what the server has done so far: residency and continuous batching */
typedef struct tdda_server_counters {
    unsigned long long operators_built;    /* cores built (each builds its Green spectrum) */
    unsigned long long operator_hits;      /* requests whose operator was resident */
    unsigned long long operators_evicted;  /* idle resident operators freed for admission */
    unsigned long long shapes_built;       /* FP32+refine: grid-shape sessions created */
    unsigned long long joined_running;     /* FP32+refine: requests admitted while others ran */
    unsigned long long rounds;             /* FP32+refine: session rounds (one launch of the steps each) */
    int max_slots_in_use;                  /* most right-hand sides sharing one launch */
    int max_lattices_in_use;               /* most different lattices sharing one launch */
    int resident_operators;                /* operators resident now */
} tdda_server_counters;
tdda_status tdda_server_counters_get(tdda_server* server, tdda_server_counters* out);
/* finishes every submitted request, then stops the workers and frees the
 * resident operators */
tdda_status tdda_server_destroy(tdda_server* server);
/* device bytes a request of nrhs right-hand sides holds while it is solved */
double tdda_request_bytes(int Nx, int Ny, int Nz, int N, int nrhs, int precision);

/* FFT engine ------------------------------------------------------------ */
/* In-place unnormalised 3-D complex128 FFT of a device array (n0, n1, n2),
 * last index fastest, sign -1 forward / +1 inverse, each n 7-smooth; the
 * engine the A-product runs on (cufftExecZ2Z's role, AProductCore.cpp:719). */
tdda_status tdda_fft3d(double* data, int n0, int n1, int n2, int sign);

/* allocation-free product (no counterpart in the reference) ------------- */
/* y = A_offdiag b in FP64 for callers that cannot allocate device memory at
 * the point of the call (memory pre-reserved under a fixed budget, or a host
 * framework that forbids allocation after its setup).  b and y are 3N complex
 * in device memory.  The FFT work grid is a static 64 MiB device array that
 * every GPU loading the library holds until exit, so the core's grid
 * 3 x Nx x My x Mz must be at most 4,194,304 complex128 entries, else
 * TDDA_ERR_UNSUPPORTED.  The product runs on the core's own stream
 * (tdda_core_stream) and the call returns when it has finished; like
 * tdda_aproduct with TDDA_MEM_DEVICE, it does not wait for other streams, so
 * the work that produces b must have finished on the device before the call
 * (a cudaStreamSynchronize of the producer's stream, or an event the core's
 * stream waits on).  The call synchronises the core's stream, so it cannot be
 * captured into a CUDA graph.  The first call on a device looks the array's
 * device address up (cudaGetSymbolAddress, which may load the library's
 * module): that first call must not overlap a global-mode stream capture in
 * another thread.  The address is kept for the life of the process, so this
 * entry point must not be used after a cudaDeviceReset of that device (the
 * reset also invalidates every core made before it).  All calls share the
 * array, so calls that overlap on the GPU (two threads, or two cores on
 * different streams) race; each call fully rewrites what it reads, so nothing
 * needs clearing between calls. */
tdda_status tdda_aproduct_noalloc(tdda_core* core, const double* b, double* y);

/* measurement hooks (no counterpart in the reference) ------------------- */
/* The CUDA stream (cudaStream_t) all work of this core runs on. */
tdda_status tdda_core_stream(const tdda_core* core, void** stream);
/* Kernels this library has launched in this process (graph replays included). */
unsigned long long tdda_kernel_launches(void);
/* Average device time in ms of each of the five A-product passes (z forward,
 * y forward, x forward + spectral product + x inverse, y inverse, z inverse)
 * over `reps` plain products of nrhs right-hand sides, timed with CUDA events
 * on the core's stream. */
tdda_status tdda_profile_aproduct(tdda_core* core, int precision, int nrhs, int reps, double* ms5);
/* Kernels of one A-product at this precision: 5 (the passes above) or 3, when
 * the z and y passes are fused (FP32 on the compiled plane sizes).  With 3,
 * tdda_profile_aproduct reports the fused forward kernel in ms5[0], the fused
 * inverse in ms5[3], and ms5[1], ms5[4] hold only the gap between two events.
 * -1 for an invalid argument. */
int tdda_core_pass_count(const tdda_core* core, int precision);
/* Kernel that runs pass `pass` (0..4, the slots of tdda_profile_aproduct) at
 * this precision: "k_zfwd", "k_ypass", "k_xpass", "k_zinv", or with the
 * fused and register forms "k_zyfwd", "k_xpass2", "k_yzinv"; "" for a slot
 * that a fused kernel covers; NULL for an invalid argument.  Static string. */
const char* tdda_core_pass_name(const tdda_core* core, int precision, int pass);

/* The FP32 x pass (x FFT, spectral product, inverse x FFT) of a core runs in
 * one of two forms: the register form on a two-stage radix plan (k_xpass2;
 * compiled for x lengths 32-192) with 8 or 16 z-columns a block, or the
 * shared-memory form on the length's compiled plan (k_xpass).  The tile does
 * not change results; the form changes the FFT's rounding (FP32 level).
 * form 0: register form where compiled, tile 8, 16 or 0 (built-in: 16 for
 * x length 128, else 8); form 1: shared-memory form, tile 0.  Captured FP32
 * solve steps of the core are dropped and captured again on next use; the
 * call waits for the core's stream first. */
tdda_status tdda_core_set_xpass(tdda_core* core, int form, int tile);
typedef struct {
    int x_form, x_tile;  /* the chosen configuration (now set on the core) */
    int ncand;           /* candidates timed: 3, or 1 where the x length has no register form */
    int form[4], tile[4];
    double ms[4];        /* average ms of one FP32 A-product of nrhs right-hand sides, per candidate */
} tdda_xpass_tune;
/* Autotuner of the FP32 x pass: times `reps` plain FP32 A-products of nrhs
 * right-hand sides (CUDA events on the core's stream, after one warm-up) for
 * every candidate form and tile, and sets the fastest on the core. */
tdda_status tdda_core_autotune(tdda_core* core, int nrhs, int reps, tdda_xpass_tune* out);

/* Batch schedule of the FP32 products of a batched solve (no counterpart in the
 * reference, which solves one right-hand side at a time): `group` right-hand
 * sides per launch, 0 for the whole batch in one launch per pass.  With groups,
 * each group runs through all of its passes before the next one starts, so the
 * FFT work grid of a group that fits in L2 stays there between the passes.
 * Results do not change (every right-hand side is computed independently).
 * Captured FP32 solve steps of the core are dropped and captured again on next
 * use; the call waits for the core's stream first.  0 <= group <= max_rhs. */
tdda_status tdda_core_set_batch_group(tdda_core* core, int group);
typedef struct {
    int group;           /* the chosen right-hand sides per launch (0: all; now set on the core) */
    int ncand;           /* candidates timed: 0, nrhs / 2, nrhs / 4, ... (at most 4) */
    int groups[4];
    double ms[4];        /* average ms of one FP32 A-product of nrhs right-hand sides, per candidate */
} tdda_batch_tune;
/* Autotuner of the batch schedule: times `reps` plain FP32 A-products of nrhs
 * right-hand sides (CUDA events, after one warm-up) for each candidate group
 * size and sets the fastest on the core. */
tdda_status tdda_core_autotune_batch(tdda_core* core, int nrhs, int reps, tdda_batch_tune* out);

#ifdef __cplusplus
}
#endif

#endif
