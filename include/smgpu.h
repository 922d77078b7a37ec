/*
 * smgpu.h — C ABI of libsmgpu.so, a GB300 (sm_103a) M-scheme shell-model
 * eigensolver that drops in for NuclearToolkit.jl's `main_sm` path.
 *
 * Every entry point is plain C: opaque handles, plain pointers and sizes,
 * integer status codes.  Each declaration names the reference interface it
 * replaces (paths relative to the NuclearToolkit.jl source tree).
 *
 * Conventions
 *  - Basis order is the reference's: block-major over (Mp,Mn) blocks ordered
 *    by ascending proton M, proton-major inside a block
 *    (M = tdims[b] + p*nn[b] + n, 0-based), Slater determinants in descending
 *    bit-string order (m-state 1 = most significant bit).
 *  - Host buffers are owned by the caller; device memory is owned by the
 *    handle.  One handle is used by one host thread at a time; different
 *    handles are independent.
 *  - Status: 0 = success, negative = error class.  smgpu_last_error() gives
 *    the message of the last failure on that handle (or of the last failed
 *    create call when given NULL).
 */
#ifndef SMGPU_H
#define SMGPU_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct smgpu_problem smgpu_problem;

enum smgpu_status_code {
  SMGPU_OK = 0,
  SMGPU_ERR_ARG = -1,       /* invalid argument */
  SMGPU_ERR_IO = -2,        /* cannot read the interaction file */
  SMGPU_ERR_PARSE = -3,     /* malformed snt content */
  SMGPU_ERR_NUCLEUS = -4,   /* nucleus name / valence numbers invalid */
  SMGPU_ERR_CUDA = -5,      /* CUDA runtime error (no device, launch failure, ...) */
  SMGPU_ERR_NOMEM = -6,     /* host or device allocation failed */
  SMGPU_ERR_LIMIT = -7,     /* problem exceeds a table-packing limit */
  SMGPU_ERR_NOCONV = -8,    /* Lanczos stopped at max_restarts before convergence */
  SMGPU_ERR_EMPTY = -9,     /* M-scheme dimension is zero */
  SMGPU_ERR_DEVICE = -10    /* a device-side check failed (bounded wait or bounds guard) */
};

/* Arithmetic of the H·v and of the Krylov basis storage. */
enum smgpu_precision {
  SMGPU_FP64 = 0,     /* plain form: everything FP64 */
  SMGPU_MIXED = 1,    /* H·v and Krylov storage FP32 (FP32 products and partial sums, the
                         partial sums of a row combined with Kahan compensation); the Lanczos
                         residual, α/β, both re-orthogonalisation passes, the restart's
                         tridiagonal/arrowhead eigensolve (FP64 Jacobi started from an FP32
                         Jacobi's eigenbasis), its Gram matrix and Cholesky factor, and the
                         Ritz vectors FP64.  The restart's basis rotation and update (whose
                         results are stored in FP32) run in compensated FP32. */
  SMGPU_MIXED_DF = 2  /* as SMGPU_MIXED, except that the residual, the re-orthogonalisation,
                         the restart eigensolve, Gram matrix and Cholesky factor run in
                         double-float arithmetic (pairs of FP32 numbers, about 48 significant
                         bits) on the FP32 pipe instead of FP64 */
};

/* Orbits are given as in an snt file: n, l, 2j, 2tz (tz = -1 proton, +1 neutron). */
typedef struct {
  int lp, ln;                /* number of proton / neutron orbits */
  const int* orbits;         /* (lp+ln) x 4 : n, l, 2j, tz — protons first */
  const double* spe;         /* lp+ln single-particle energies */
  int ntbme;                 /* number of TBME entries below */
  const int* tbme_labels;    /* ntbme x 5 : a, b, c, d (1-based orbit index), J */
  const double* tbme;        /* ntbme values, massop scaling already applied */
  int hermitian_partners;    /* 1: add (c,d,a,b) for every {a,b}!={c,d} entry as readsmsnt does */
  int vp, vn;                /* valence protons / neutrons */
  int mtot2;                 /* doubled total M */
} smgpu_problem_desc;

/* Parse an snt file and set the problem up as main_sm does for target_J = []:
 * readsmsnt (src/ShellModel/shellmodel_main.jl:293-365), mass number and
 * element from the nucleus name (util_func.jl:1,13-24; shellmodel_main.jl:
 * 95,116-117,908-916), Mtot = A mod 2 (:110), basis and jump tables
 * (occ :769-848, prep_Hamil_T1 :580-649, prep_Hamil_pn :658-730,
 * prep_pn :1139-1199): the basis and the jump tables are enumerated on the
 * GPU, the interaction's operator lists on the host. */
int smgpu_problem_create_from_snt(const char* snt_path, const char* nucleus, int precision, smgpu_problem** out);

/* Same for main_sm with target_J = [twoJ/2]: the basis has Mtot = twoJ
 * (shellmodel_main.jl:112-116); twoJ must have the parity of A
 * (SMGPU_ERR_NUCLEUS otherwise). */
int smgpu_problem_create_from_snt_J(const char* snt_path, const char* nucleus, int twoJ, int precision,
                                    smgpu_problem** out);

/* Same, from an in-memory description (the data of the reference's SMobject,
 * shellmodel_main.jl:38-53). */
int smgpu_problem_create(const smgpu_problem_desc* desc, int precision, smgpu_problem** out);

/* Free all device and host memory of the handle. */
int smgpu_problem_destroy(smgpu_problem* h);

/* Message of the last failure (handle-owned string; NULL handle = last create failure). */
const char* smgpu_last_error(const smgpu_problem* h);

/* M-scheme dimension and block table (the reference's mdim = tdims[end] and
 * tdims, shellmodel_main.jl:126-128).  tdims_out may be NULL, else holds
 * nblocks+1 entries. */
int smgpu_dims(const smgpu_problem* h, long long* mdim, int* nblocks, long long* tdims_out);

/* Per-block data: proton/neutron SD counts and M values (each array nblocks
 * long, any may be NULL).  Replaces pbits/nbits lengths and Mps/Mns of occ. */
int smgpu_blocks(const smgpu_problem* h, int* np, int* nn, int* mp2, int* mn2);

/* Copy the proton and neutron Slater determinants (bit strings, blocks
 * concatenated in order) to host buffers of sum(np) and sum(nn) entries. */
int smgpu_export_basis(const smgpu_problem* h, unsigned long long* pbits, unsigned long long* nbits);

/* Jump tables in the reference's forward form for parity checks.
 * which = 0: proton one-body pn jumps, 1: neutron one-body pn jumps,
 *         2: pp two-body jumps, 3: nn two-body jumps.
 * count: number of entries.  For which 0/1 each entry is
 *   (bi, bf, op_a, op_c, i, f, phase) with op bits as the reference's bit2b
 *   masks, 1-based block and SD indices, phase = 1 for an odd permutation count;
 * for which 2/3: (block, i, f) and the coefficient in `coef` (f >= i, the
 * reference's T1info with the 1/2 on the diagonal).
 * Call with NULL buffers to get the count. */
int smgpu_export_jumps(const smgpu_problem* h, int which, long long* count, long long* ints, double* coef);

/* w (+)= H v on host buffers in the reference's basis order (unpadded, mdim
 * doubles each, ncols column vectors stored one after another).
 * accumulate = 1 reproduces operate_H!'s "twf += H wf" (lanczos_methods.jl:153);
 * accumulate = 0 overwrites w.  Runs in the handle's precision. */
int smgpu_matvec(smgpu_problem* h, const double* v, double* w, int ncols, int accumulate);

/* Thick-restart Lanczos for the lowest num_ev eigenvalues: TRL with
 * diagonalize_T!/ThickRestart (lanczos_methods.jl:1-91,250-307) and Ritz
 * vectors (shellmodel_main.jl:208-224), entirely on the GPU.
 *   lm, ls, tol: as main_sm's kwargs (defaults 300, 20, 1e-8);
 *   max_restarts: stop with SMGPU_ERR_NOCONV after this many restarts;
 *   v1: optional start vector (mdim doubles, host), NULL = seeded hash draw;
 *   evals_out: num_ev doubles (min(num_ev, mdim) are written);
 *   evecs_out: NULL or num_ev x mdim doubles (Ritz vectors, basis order);
 *   stats_out: NULL or 8 ints: [elit, n_matvec, n_restart, converged, num_ev_written,
 *              second re-orthogonalisation passes, kernel launches, reserved]. */
int smgpu_solve(smgpu_problem* h, int num_ev, int lm, int ls, double tol, int max_restarts,
                const double* v1, double* evals_out, double* evecs_out, int* stats_out);

/* <v|J^2|v>/<v|v> for nvec host vectors (mdim doubles each, basis order):
 * the expectation values main_sm prints as J labels (operate_J! on the Ritz
 * vectors and J_from_JJ1, shellmodel_main.jl:226-240,1105-1113).  J^2 is
 * applied on the GPU in FP64 as an operator on the same basis (built on the
 * first call from the handle's orbits: one-body j(j+1), two-body
 * J(J+1) - j_a(j_a+1) - j_b(j_b+1) per pair). */
int smgpu_jj(smgpu_problem* h, const double* vecs, int nvec, double* jj_out);

/* One-body electromagnetic operators of transit.jl. */
enum { SMGPU_OBTR_M1 = 0, SMGPU_OBTR_E2 = 1 };

/* out[a*nr + b] = <vl_a| O |vr_b> for the M1 (op = SMGPU_OBTR_M1) or E2
 * (SMGPU_OBTR_E2) one-body operator, vl_a nl host vectors of hl's basis and
 * vr_b nr host vectors of hr's basis (reference order).  symmetric != 0 is
 * the expectation-value form of eval_moment (prep_obtr_diag / op_obtr_diag,
 * src/ShellModel/transit.jl:82-284,702-765: orbit pairs f >= i applied with
 * their transpose; hl and hr share one basis); symmetric == 0 is
 * transit_main's (prep_obtr_nondiag / op_obtr_nondiag / calc_bifs,
 * :286-531,561-700) with ΔM = (Mtot_l - Mtot_r)/2 (doubled Mtot of the
 * handles; the reference takes Mtot_l >= Mtot_r).  gfactors = [g_l(p),
 * g_l(n), g_s(p), g_s(n)] (NULL: 1.0, 0.0, 5.586, -3.826), effcharge =
 * [e_p, e_n] (NULL: 1.5, 0.5); the oscillator length follows
 * init_ho_by_mass (hwprm 2 for 16 <= A <= 40).  O·v and the overlaps run on
 * the GPU in FP64; nl * nr <= 65535.  Both handles must describe one nucleus
 * on one model space (SMGPU_ERR_ARG). */
int smgpu_obtr(smgpu_problem* hl, smgpu_problem* hr, int op, int symmetric, const double* gfactors,
               const double* effcharge, const double* vl, int nl, const double* vr, int nr, double* out);

/* Transition densities of eigenvector continuation (prepEC mode "TD",
 * src/ShellModel/eigenvector_continuation.jl:212-310; calcOBTD, prepTBTD,
 * calcTBTD :1035-1380) for nvec sample vectors of h's basis (host, reference
 * order, nvec <= 255): nmat_out[i*nvec + j] = <w_i|w_j>, and for each pair
 * i <= j, in idx_from_ij order (shellmodel_main.jl:1297), ltd values
 * td_out[pair*ltd + u]: the derivatives of <w_i|H|w_j> with respect to the
 * proton SPEs (u < lp), the neutron SPEs, and the value of each TBME line of
 * the snt file the handle was created from (hermitian partner included, no
 * mass scaling) — the reference's OBTD and TBTD.  ltd = lp + ln + number of
 * TBME lines (smgpu_ec_td_length).  Every unit's Hamiltonian is set up on
 * the sample basis and applied on the GPU in FP64. */
int smgpu_ec_td_length(const smgpu_problem* h, int* ltd);
int smgpu_ec_td(smgpu_problem* h, const double* vecs, int nvec, double* nmat_out, double* td_out);

/* Wigner 3j (j1 j2 j3; m1 m2 m3) and 6j {j1 j2 j3; j4 j5 j6} symbols with
 * doubled arguments (the values of WignerSymbols.jl's wigner3j / wigner6j,
 * used by eval_moment and transit_main; host code, no GPU needed). */
double smgpu_wigner3j(int tj1, int tj2, int tj3, int tm1, int tm2, int tm3);
double smgpu_wigner6j(int tj1, int tj2, int tj3, int tj4, int tj5, int tj6);

/* J-projected ("double") Lanczos for the lowest num_ev states of total
 * angular momentum twoJ/2: TRL with doubleLanczos = true
 * (lanczos_methods.jl:1-91) — every new Krylov vector is projected onto J by
 * an inner Lanczos on J^2 (Jlanczos / ThickRestart_J, :93-151, tolerance
 * 1e-7 on J(J+1)) and re-orthogonalised.  The handle must come from
 * smgpu_problem_create_from_snt_J with the same twoJ; ls >= 2 (it is also
 * the length of the inner Lanczos).  Arguments and outputs as smgpu_solve;
 * J^2 is built on the first call (as smgpu_jj).  Runs in FP64 for either
 * precision of the handle (FP32 Krylov vectors hold rounding components of
 * every J, from which lower-lying states of other J re-emerge). */
int smgpu_solve_J(smgpu_problem* h, int twoJ, int num_ev, int lm, int ls, double tol, int max_restarts,
                  const double* v1, double* evals_out, double* evecs_out, int* stats_out);

/* Block thick-restart Lanczos, main_sm's is_block = true with block size q
 * (TRBL, lanczos_methods.jl:312-423, bl_QR!, bl_ReORTH, add_bl_T!,
 * bl_ThickRestart): blocks of q vectors, ls/q kept blocks at a restart, the
 * block T diagonalised every iteration; FP64 for either handle precision.
 * v1: NULL (q seeded hash draws, seeds 1234..1234+q-1, orthonormalised) or
 * q x mdim; stats_out[1] counts single-vector H·v; stats_out[7] = q.  Other
 * arguments and outputs as smgpu_solve. */
int smgpu_solve_block(smgpu_problem* h, int q, int num_ev, int lm, int ls, double tol, int max_restarts,
                      const double* v1, double* evals_out, double* evecs_out, int* stats_out);

/* Seconds spent in the phases of the last create / solve / matvec call (the
 * reference's TimerOutputs sections "prep. 1b&2b-jumps", "Lanczos", "Rvecs",
 * shellmodel_main.jl:137,159,208).  times_out: 8 doubles:
 * [setup (host wall), lanczos (CUDA events on the handle's stream, start
 *  vector to converged eigenvalues), last matvec call (host wall), graph
 *  capture + instantiation (host wall), ritz vectors (events), solve call
 *  (host wall), set-up part: basis and jump tables (host wall), set-up
 *  part: device tables, staged-kernel tables and autotuning (host wall)]. */
int smgpu_timings(const smgpu_problem* h, double* times_out);

/* Time `reps` back-to-back H·v launches on the handle's stream with CUDA
 * events (the reference's "operate H" section, lanczos_methods.jl:36), on a
 * device-resident seeded vector in the handle's precision.  flush_l2 != 0
 * writes a 256 MB buffer between launches and excludes that from the time.
 * ms_out: mean milliseconds per launch. */
int smgpu_time_matvec(smgpu_problem* h, int reps, int flush_l2, double* ms_out);

/* Read bandwidth (GB/s) of a device buffer of `bytes` (1 MB .. 1 GB) that
 * stays resident in the L2 cache: `reps` launches of the library's own read
 * kernel, 16 sweeps over the buffer each, timed with CUDA events after one
 * untimed sweep.  No
 * counterpart in the reference: the ceiling against which the H·v kernels,
 * whose tables and vectors fit in L2, are measured. */
int smgpu_l2_read_bandwidth(long long bytes, int reps, double* gbs_out);

/* The H·v autotuner's measurements for this handle (no counterpart in the
 * reference, whose operate_H! has one form): *count = number of candidate
 * launch shapes timed when the handle was created (0 when the shape came
 * from the cache or SMGPU_AUTOTUNE=0); for the first min(max, *count) of
 * them, shapes[4k..4k+3] = (threads per CTA, rows per CTA, minimum CTAs per
 * SM, kernel form: 0 row-tile, 1 staged pn) and ms[k] = mean ms per launch
 * (for a shape dropped because its warm-up launch took more than twice the
 * best mean so far: that warm-up launch's time).  Staged shapes are timed
 * first. */
int smgpu_tune_report(const smgpu_problem* h, int max, int* shapes, double* ms, int* count);

/* Structural statistics of the factorised H (12 entries): [updates per H·v
 * (multiply-adds), pn proton pull entries, pn neutron entries, pp entries,
 * nn entries, table bytes on the device, padded vector length, number of
 * links, H·v threads per CTA, H·v rows per CTA, H·v minimum CTAs per SM,
 * H·v kernel form (0 row-tile, 1 staged pn) — the last four the autotuned
 * launch shape]. */
int smgpu_stats(const smgpu_problem* h, long long* stats_out);

/* H·v that allocates nothing.  No counterpart in the reference: it exists for
 * callers whose device memory is owned by their own pool allocator (a Julia
 * CuArray pool, PyTorch's caching allocator).  Such a pool usually holds most
 * of the device's memory, so a library's cudaMalloc in the middle of a step
 * can fail or force the pool to release its cache, and a cudaFree
 * synchronizes the whole device, stalling the host's queued work.
 *   v, w : caller-owned DEVICE buffers of mdim doubles in the reference's
 *          basis order (the layout of smgpu_matvec's host vectors);
 *          w = H v is overwritten, the FP64 form is used;
 *   vhv  : NULL or a caller-owned DEVICE double that receives <v|H|v>.
 * The only scratch, the per-CTA partial sums of <v|H|v>, is a file-scope
 * device array of 65,536 doubles (512 KB) that every GPU loading the library
 * holds until exit; problems whose H·v launch has more CTAs than that, and
 * handles created with a mixed precision, are rejected (SMGPU_ERR_LIMIT /
 * SMGPU_ERR_ARG).  The first call on a device looks up the array's device
 * address and caches it for the process (cudaDeviceReset between calls is
 * not supported).  The kernels run on the handle's own stream, which is not
 * ordered with the caller's streams: all device work writing v must be
 * finished before the call (e.g. by a stream or device synchronize); the call
 * returns when w and *vhv are ready.  All calls share the array (each call
 * rewrites every entry it reads), so calls that overlap on the GPU race. */
int smgpu_matvec_noalloc(smgpu_problem* h, const double* v, double* w, double* vhv);

/* ------------------------------------------------------------------------
 * `.wav` files (writeRitzvecs / read_wav / read_appwav,
 * src/ShellModel/shellmodel_main.jl:967-1003,1215-1229): int32 neig, int32
 * Mtot (doubled), float64 E[neig], int32 2J[neig], float64 V[neig][mdim],
 * native little-endian.  Host-only calls (no GPU needed); errors are
 * reported by smgpu_wav_last_error(). */
int smgpu_write_wav(const char* path, long long mdim, int mtot2, int nev, const double* evals, const int* twoJ,
                    const double* vecs);
/* Number of vectors and Mtot of a file whose size matches dimension mdim. */
int smgpu_read_wav_header(const char* path, long long mdim, int* nev, int* mtot2);
/* The first min(neig, nev_max) energies, 2J labels and vectors (any output
 * may be NULL). */
int smgpu_read_wav(const char* path, long long mdim, int nev_max, double* evals, int* twoJ, double* vecs);
const char* smgpu_wav_last_error(void);

/* ------------------------------------------------------------------------
 * Interaction samples sharing one basis (the sample loop of prepEC,
 * src/ShellModel/eigenvector_continuation.jl:102-312: one snt per sample,
 * the basis of the first, TRL per sample).  Up to 16 samples are solved
 * together in the FP32-mixed form: one multi-sample H·V per Lanczos
 * iteration reads the shared jump tables once for all samples; every sample
 * keeps its own Lanczos matrix, convergence test and thick restart.
 * Vectors on the host are sample-major: sample s at [s*mdim, (s+1)*mdim). */
typedef struct smgpu_multi smgpu_multi;

/* Read nsamples snt files (1..16) for one nucleus.  The samples must give the
 * same valence space and the same non-zero pattern of m-scheme matrix
 * elements (SMGPU_ERR_LIMIT otherwise).  Replaces the per-sample readsmsnt,
 * prep_Hamil_T1, prep_Hamil_pn and prep_pn calls of prepEC (:140-153). */
int smgpu_multi_create_from_snt(const char* const* snt_paths, int nsamples, const char* nucleus,
                                smgpu_multi** out);
int smgpu_multi_destroy(smgpu_multi* h);
/* Message of the last failure on h (NULL: of the last failed create call). */
const char* smgpu_multi_last_error(const smgpu_multi* h);
/* mdim, number of samples, and the lane count S the kernels run with
 * (4, 8 or 16; samples beyond nsamples are idle lanes). */
int smgpu_multi_dims(const smgpu_multi* h, long long* mdim, int* nsamples, int* lanes);

/* w_s (+)= H_s v_s for every sample s (operate_H! per sample,
 * lanczos_methods.jl:153), host buffers of nsamples x mdim doubles. */
int smgpu_multi_matvec(smgpu_multi* h, const double* v, double* w, int accumulate);

/* TRL for the lowest num_ev eigenvalues of every sample (prepEC's per-sample
 * TRL call, eigenvector_continuation.jl:171-177, without J projection).
 *   lm, ls, tol, max_restarts: as smgpu_solve (one value for all samples);
 *   v1: NULL (seeded hash draw, the same for every sample) or nsamples x mdim;
 *   evals_out: nsamples x num_ev doubles (en[1] of each sample's last test);
 *   evecs_out: NULL or nsamples x num_ev x mdim (Ritz vectors of the
 *              converged samples);
 *   stats_out: NULL or 8 + 4*nsamples ints: [multi-sample H·V launches,
 *              restarts, all converged, num_ev written, kernel launches,
 *              lanes, reserved, reserved], then per sample [elit, converged,
 *              second re-orthogonalisation passes, reserved].
 * Returns SMGPU_ERR_NOCONV when some sample has not converged after
 * max_restarts restarts (the other samples' results are still written). */
int smgpu_multi_solve(smgpu_multi* h, int num_ev, int lm, int ls, double tol, int max_restarts,
                      const double* v1, double* evals_out, double* evecs_out, int* stats_out);

/* Statistics (8 entries): [multiply-adds per sample per H·V, lanes, device
 * table bytes (shared structure + interleaved coefficients), padded vector
 * length, H·V CTAs, and the autotuned launch shape: threads per CTA, minimum
 * CTAs per SM, neutron entries cached in registers]. */
int smgpu_multi_stats(const smgpu_multi* h, long long* stats_out);

/* As smgpu_timings, for the last create / solve / matvec call on h. */
int smgpu_multi_timings(const smgpu_multi* h, double* times_out);

/* Mean milliseconds of one multi-sample H·V launch over `reps` launches on a
 * device-resident seeded vector (flush_l2 as smgpu_time_matvec). */
int smgpu_multi_time_matvec(smgpu_multi* h, int reps, int flush_l2, double* ms_out);

/* ------------------------------------------------------------------------
 * Batches of independent problems (many main_sm calls,
 * src/ShellModel/shellmodel_main.jl:89-281, each with its own snt file and
 * nucleus, so each its own basis and dimension).  The batch is solved in the
 * FP32-mixed form with every launch covering all problems: one H·v launch
 * over the row tiles of every problem, the re-orthogonalisation over chunks
 * of the concatenated vectors, one CTA per problem for the small kernels;
 * the H·v launch shape is autotuned on the whole batch.  Host vectors are
 * the problems' vectors (reference basis order) concatenated in problem
 * order: problem p at [moff_p, moff_p + mdim_p), moff_p = sum of the earlier
 * problems' dimensions. */
typedef struct smgpu_batch smgpu_batch;

/* nprob (1..4096) snt files and nuclei; problem p is main_sm's set-up of
 * (snt_paths[p], nuclei[p]) for target_J = [] (readsmsnt, occ, prep_Hamil_T1,
 * prep_Hamil_pn, prep_pn: shellmodel_main.jl:95-147). */
int smgpu_batch_create_from_snt(const char* const* snt_paths, const char* const* nuclei, int nprob,
                                smgpu_batch** out);
int smgpu_batch_destroy(smgpu_batch* h);
const char* smgpu_batch_last_error(const smgpu_batch* h);
/* Sum of the dimensions, number of problems, and (NULL or nprob entries) the
 * dimension of every problem. */
int smgpu_batch_dims(const smgpu_batch* h, long long* total_mdim, int* nprob, long long* mdims);

/* w (+)= H_p v_p for every problem (operate_H!, lanczos_methods.jl:153), host
 * buffers of total_mdim doubles (concatenated problem vectors). */
int smgpu_batch_matvec(smgpu_batch* h, const double* v, double* w, int accumulate);

/* TRL for the lowest num_ev eigenvalues of every problem (lanczos_methods.jl:
 * 1-91 with diagonalize_T!/ThickRestart, :250-307), all problems together.
 *   lm, ls, tol, max_restarts: as smgpu_solve (one value for all problems);
 *   v1: NULL (seeded hash draw per problem) or total_mdim doubles;
 *   evals_out: nprob x num_ev doubles; problem p's entries beyond
 *              min(num_ev, mdim_p) are NaN;
 *   evecs_out: NULL or num_ev x total_mdim doubles: problem p's Ritz vectors
 *              at [num_ev*moff_p, num_ev*(moff_p + mdim_p)), one mdim_p run
 *              per eigenvalue (zeros for unconverged problems);
 *   stats_out: NULL or 8 + 4*nprob ints: [batched H·v launches, restarts, all
 *              converged, num_ev, kernel launches, problems, chunks, H·v
 *              tasks], then per problem [elit, converged, second
 *              re-orthogonalisation passes, reserved].
 * Returns SMGPU_ERR_NOCONV when some problem has not converged after
 * max_restarts restarts (the results of all problems are still written). */
int smgpu_batch_solve(smgpu_batch* h, int num_ev, int lm, int ls, double tol, int max_restarts,
                      const double* v1, double* evals_out, double* evecs_out, int* stats_out);

/* Statistics (9 entries): [multiply-adds per batched H·v, problems, chunks,
 * H·v tasks, and the autotuned launch shape: threads per CTA, rows per CTA,
 * minimum CTAs per SM; device table bytes; 1 when that shape is the staged
 * pn form]. */
int smgpu_batch_stats(const smgpu_batch* h, long long* stats_out);

/* As smgpu_timings, for the last create / solve / matvec call on h. */
int smgpu_batch_timings(const smgpu_batch* h, double* times_out);

/* Mean milliseconds of one batched H·v launch (all problems) over `reps`
 * launches on a device-resident seeded vector (flush_l2 as smgpu_time_matvec). */
int smgpu_batch_time_matvec(smgpu_batch* h, int reps, int flush_l2, double* ms_out);

#ifdef __cplusplus
}
#endif
#endif /* SMGPU_H */
