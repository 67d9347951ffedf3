/*
 * qtt_gb300.h -- C-ABI of the GB300 block-sparse tensor library (libqtt_gb300.so).
 *
 * This is the drop-in boundary for QuantiT's block-sparse hot path: btensor
 * contraction (tensordot / tensorgdot), per-charge-sector SVD / eigh with
 * truncation, and the two-site DMRG update (Heff*theta matvec, one-step Lanczos,
 * 2x2 Ritz solve) with its sweep driver.  Each entry point names the QuantiT
 * interface it replaces (paths relative to the QuantiT source tree).
 *
 * Conventions
 *  - Every function returns an int status (QTT_OK == 0).  On failure the message
 *    is available from qtt_last_error() (thread local).  The status names the C++
 *    exception QuantiT throws for the same condition.
 *  - A btensor is an opaque handle (qtt_bt).  Results are new handles owned by
 *    the caller and released with qtt_bt_destroy.  Handles are immutable once
 *    created, except through the explicitly in-place calls (qtt_tensorgdot_ and
 *    qtt_bt_set_blocks*).
 *  - Charges: a group has `ncomp` factors (<= 4); moduli[i] == 0 marks a U(1)
 *    factor (QuantiT conserved::Z, int16 addition), moduli[i] == N > 0 a Z(N)
 *    factor (conserved::C<N>, addition mod N).  A charge is `ncomp` int16 values;
 *    arrays of charges are packed [n][ncomp].
 *  - Block data is dense row-major per block; blocks are concatenated in the
 *    order of the block list (lexicographic in the block index, like QuantiT's
 *    flat_map, unless a call documents otherwise).
 *  - All device work is issued on the calling thread's current stream
 *    (qtt_set_stream; default: a stream the library creates).
 *  - dtype: QTT_F64 (the drop-in) or QTT_F32.
 */
#ifndef QTT_GB300_H
#define QTT_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct qtt_bt_s *qtt_bt;

enum {
    QTT_OK = 0,
    QTT_ERR_INVALID_ARGUMENT = 1, /* std::invalid_argument */
    QTT_ERR_OUT_OF_RANGE = 2,     /* std::out_of_range */
    QTT_ERR_DOMAIN = 3,           /* std::domain_error */
    QTT_ERR_LOGIC = 4,            /* std::logic_error */
    QTT_ERR_RUNTIME = 5,          /* std::runtime_error */
    QTT_ERR_CUDA = 6,             /* CUDA runtime failure */
    QTT_ERR_OOM = 7,              /* device allocation failure */
    QTT_ERR_CHECK = 8,            /* c10::Error (TORCH_CHECK in the reference) */
    QTT_ERR_NO_DATA = 9           /* structure-only btensor given to a numeric call */
};
enum { QTT_F64 = 0, QTT_F32 = 1 };
/* precision of the block GEMMs (tensordot / matvec): FP64, or split TF32 (hi/lo) or
 * split BF16 (hi/mid/lo) on the tensor cores with FP32 accumulation.  Under a split
 * mode the sector SVD runs its first sweeps in FP32 and finishes them in FP64 (an FP64
 * SVD either way); eigh, inner products, norms and the 2x2 solve always run in FP64. */
enum { QTT_GEMM_F64 = 0, QTT_GEMM_TF32X3 = 1, QTT_GEMM_BF16X3 = 2 };

/* ------------------------------------------------------------------ library */
const char *qtt_last_error(void);
const char *qtt_version(void);
/* Select the CUDA device for the calling thread and create its default stream. */
int qtt_init(int device);
/* Use `stream` (a cudaStream_t) for the calling thread's work; NULL restores the default. */
int qtt_set_stream(void *stream);
void *qtt_get_stream(void);
int qtt_synchronize(void);
/* Block-GEMM precision for the calling process (QTT_GEMM_*). */
int qtt_set_gemm_mode(int mode);
int qtt_get_gemm_mode(void);
/* Block-width autotuner of the sector-SVD kernel (no reference counterpart): on by
 * default; the first decompositions of each class (precision, column length, widest
 * sector, sector count) time the candidate widths and keep the faster.
 * QTT_AUTOTUNE_FILE persists the decisions.  The report lists them, one per line;
 * *len receives its length. */
int qtt_set_autotune(int on);
int qtt_autotune_report(char *buf, int64_t cap, int64_t *len);
/* Deflation in the sector SVD of a truncating svd (no reference counterpart; on by
 * default): a column whose norm falls to the sweeps' resolution (FP32 epsilon, or 8
 * FP64 epsilons, times its sector's Frobenius norm) leaves the sweeps and keeps that
 * norm as its value, far below any value a truncation keeps; the FP64 sweeps of the
 * mixed path resolve what its FP32 sweeps dropped. */
int qtt_set_svd_deflation(int on);
/* Block-sparsity planner of tensordot / tensorgdot (the charge check and merge-join of
 * sources/btensor.cpp:783-883,1998-2110): mode 0 plans on the host, 1 on the device
 * wherever the device planner's limits allow (at most 16384 blocks per operand, keys
 * within 63 bits, at least one contracted leg), 2 on the device for contractions with
 * at least auto_blocks blocks in the two operands together (default: mode 0; auto_blocks 3000).
 * Both emit the same output block list and pair order, bit for bit.  Inside CUDA-graph
 * capture the host plans. */
int qtt_set_planner(int mode, int64_t auto_blocks);
/* Planner calls since the last reset: calls[0] on the host, calls[1] on the device,
 * calls[2] device attempts beyond its limits (planned on the host); secs[0], secs[1]:
 * host wall seconds spent planning on each path.  reset != 0 clears them. */
int qtt_planner_stats(int64_t *calls, double *secs, int reset);
/* Persistent split-TF32 / split-BF16 GEMMs (one CTA per SM walking the tile list, double-buffered TMEM
 * accumulator) for launches of at least two tiles per SM; on by default (no reference
 * counterpart). */
int qtt_set_persistent_gemm(int on);
/* Free and total bytes of the calling thread's device (no reference counterpart;
 * the serving loop admits solves against it). */
int qtt_device_memory(int64_t *free_bytes, int64_t *total_bytes);
/* Sector-SVD kernel (no reference counterpart; a tuning and testing switch):
 * 0 = block-cyclic Jacobi wherever the sector shapes fit it (default),
 * 1 = scalar Jacobi (one column pair per warp and grid step) everywhere. */
int qtt_set_jacobi_kernel(int which);

/* ------------------------------------------------------------------ btensor
 * btensor(index_list sections_by_dim, any_quantity_vector c_vals, index_list
 * section_sizes, any_quantity sel_rule, TensorOptions)
 * (include/blockTensor/btensor.h:134): an empty block list over the given legs.
 * sections_by_dim[rank], section_sizes[nsec], c_vals[nsec][ncomp], sel[ncomp]. */
int qtt_bt_create(int32_t rank, const int64_t *sections_by_dim, const int64_t *section_sizes, int32_t ncomp,
                  const uint16_t *moduli, const int16_t *c_vals, const int16_t *sel, int32_t dtype, qtt_bt *out);
/* Set the block list.  block_index[nblocks][rank]; a disallowed block fails with
 * QTT_ERR_INVALID_ARGUMENT like btensor::block (btensor.cpp:380-395).  The list
 * is sorted into flat_map order.  host_data: the blocks concatenated in the
 * order given (row-major each), or NULL for zeros.  Uploads to the device. */
int qtt_bt_set_blocks(qtt_bt t, int64_t nblocks, const int64_t *block_index, const void *host_data);
/* Same with the data already on the device (copied, device to device). */
int qtt_bt_set_blocks_device(qtt_bt t, int64_t nblocks, const int64_t *block_index, const void *device_data);
/* Block list without data: a structure-only btensor.  Structure-only tensors flow
 * through tensordot / reshape / permute / svd-structure calls without touching a
 * GPU, which lets the planner be checked on a machine without one. */
int qtt_bt_set_block_structure(qtt_bt t, int64_t nblocks, const int64_t *block_index);
int qtt_bt_destroy(qtt_bt t);
int qtt_bt_clone(qtt_bt t, qtt_bt *out); /* shares the device data */
/* Sizes of the structure tables. */
int qtt_bt_meta(qtt_bt t, int32_t *rank, int64_t *nsections, int32_t *ncomp, int64_t *nblocks, int64_t *nnz,
                int32_t *dtype, int32_t *has_data);
int qtt_bt_structure(qtt_bt t, int64_t *sections_by_dim, int64_t *section_sizes, int16_t *c_vals, int16_t *sel,
                     uint16_t *moduli);
/* block_index[nblocks][rank] in block-list order, and each block's element count. */
int qtt_bt_blocks(qtt_bt t, int64_t *block_index, int64_t *block_numel);
/* Download all blocks, concatenated in block-list order (nbytes >= nnz*itemsize). */
int qtt_bt_download(qtt_bt t, void *host, int64_t nbytes);
/* check_tensor (btensor.cpp:405-467): writes the report (empty when consistent). */
int qtt_bt_check(qtt_bt t, char *msg, int64_t cap);

/* ------------------------------------------------------------------ structure ops */
/* btensor::permute (btensor.h:555, btensor.cpp:1754) */
int qtt_permute(qtt_bt t, const int64_t *perm, qtt_bt *out);
/* btensor::reshape(index_groups) (btensor.h:569, btensor.cpp:2986) */
int qtt_reshape(qtt_bt t, int32_t ngroups, const int64_t *index_groups, qtt_bt *out);
/* btensor::reshape_as<dims_only> (btensor.h:585, btensor.cpp:3027) */
int qtt_reshape_as(qtt_bt t, qtt_bt shape, qtt_bt *out);
/* btensor::conj / inverse_cvals (btensor.h:649,669; btensor.cpp:2156-2172) */
int qtt_conj(qtt_bt t, qtt_bt *out);
int qtt_inverse_cvals(qtt_bt t, qtt_bt *out);

/* ------------------------------------------------------------------ contraction */
/* btensor::tensordot (btensor.h:623,1230; btensor.cpp:1971-2119): all
 * charge-matched block products of the contraction as one grouped GEMM. */
int qtt_tensordot(qtt_bt a, qtt_bt b, int32_t ndims, const int64_t *dims_a, const int64_t *dims_b, qtt_bt *out);
/* tensorgdot(add, mul1, mul2, dims1, dims2, beta, alpha) = beta*add + alpha*mul1.mul2
 * (declared at btensor.h:624-627,1247-1268 without a definition in QuantiT; the
 * addmm semantics of the dense tensorgdot, sources/tensorgdot.cpp:102-117). */
int qtt_tensorgdot(qtt_bt add, qtt_bt a, qtt_bt b, int32_t ndims, const int64_t *dims_a, const int64_t *dims_b,
                   double beta, double alpha, qtt_bt *out);
/* tensorgdot_ (btensor.h:626,1264): the result replaces add's blocks in place. */
int qtt_tensorgdot_(qtt_bt add, qtt_bt a, qtt_bt b, int32_t ndims, const int64_t *dims_a, const int64_t *dims_b,
                    double beta, double alpha);

/* ------------------------------------------------------------------ algebra */
/* btensor::add(other, alpha) (btensor.h:462): a + alpha*b over the union of blocks */
int qtt_add(qtt_bt a, qtt_bt b, double alpha, qtt_bt *out);
/* btensor::mul(Scalar) (btensor.h:548) */
int qtt_mul_scalar(qtt_bt a, double s, qtt_bt *out);
/* tensordot(a, b.conj(), all legs).item() for real data */
int qtt_dot_all(qtt_bt a, qtt_bt b, double *out);
/* u.mul(d) with d a rank-1 btensor broadcast on u's last leg (btensor.h:547) */
int qtt_mul_lastleg(qtt_bt u, qtt_bt d, qtt_bt *out);

/* ------------------------------------------------------------------ decompositions */
/* svd(btensor, some=true) (blockTensor/LinearAlgebra.h:74; btensor_linalg.cpp:390) */
int qtt_svd(qtt_bt t, qtt_bt *U, qtt_bt *d, qtt_bt *V);
/* svd(btensor, split) (LinearAlgebra.h:87; btensor_linalg.cpp:503) */
int qtt_svd_split(qtt_bt t, int64_t split, qtt_bt *U, qtt_bt *d, qtt_bt *V);
/* svd(A, split, tol, min_size, max_size, pow) (LinearAlgebra.h:115; btensor_linalg.cpp:805) */
int qtt_svd_truncate(qtt_bt t, int64_t split, double tol, int64_t min_size, int64_t max_size, double pow,
                     qtt_bt *U, qtt_bt *d, qtt_bt *V);
/* truncate(U, d, V, max, min, tol, pow) (LinearAlgebra.h:246; btensor_linalg.cpp:658-755) */
int qtt_truncate(qtt_bt U, qtt_bt d, qtt_bt V, int64_t max_size, int64_t min_size, double tol, double pow,
                 qtt_bt *Uo, qtt_bt *do_, qtt_bt *Vo);
/* eigh(btensor, upper) and eigh(btensor, split) (LinearAlgebra.h:159,167; btensor_linalg.cpp:294,369) */
int qtt_eigh(qtt_bt t, int32_t upper, qtt_bt *d, qtt_bt *U);
int qtt_eigh_split(qtt_bt t, int64_t split, qtt_bt *d, qtt_bt *U);

/* ------------------------------------------------------------------ DMRG (include/dmrg.h) */
typedef struct {
    double cutoff;                 /* dmrg_options::cutoff (default 1e-6) */
    double convergence_criterion;  /* relative energy change per sweep (default 1e-5) */
    int64_t maximum_bond;          /* default: unbounded */
    int64_t minimum_bond;          /* default 4 */
    int64_t maximum_iterations;    /* sweeps (default 1000) */
    int32_t gemm_mode;             /* QTT_GEMM_* for the matvecs and environment updates */
    int32_t final_energy_fp64;     /* mixed gemm_mode: use the FP64 <psi|H|psi>/<psi|psi> of the state
                                      instead of the last Ritz value -- after every sweep for the
                                      convergence test and the log when convergence_criterion > 0,
                                      and for the returned energy (default 1) */
    int32_t lanczos_steps;         /* 1: QuantiT's one-step update (two_sites_update, dmrg.cpp:624-638);
                                      k > 1: k-step Lanczos with full reorthogonalisation (no
                                      reference counterpart; default 1) */
    int32_t cuda_graphs;           /* k-step Lanczos: capture the two-site matvec once per bond as a CUDA
                                      graph and replay it for the remaining iterations (default 1) */
    int32_t svd_warm_start;        /* start each bond's sector SVD from the rotation of that bond's
                                      previous decomposition in this call (no reference counterpart;
                                      exact for any start; default 1) */
    int32_t pad;
} qtt_dmrg_options;
/* dmrg_options defaults (include/dmrg_options.h:15-58) */
void qtt_dmrg_options_default(qtt_dmrg_options *opt);
/* Called after each sweep (dmrg_logger::it_log_all, dmrg_logger.h:53): sweep
 * number, the sweep's last energy, the sweep's wall time in seconds. */
typedef void (*qtt_dmrg_log_fn)(void *user, int64_t sweep, double energy, double seconds);

/* dmrg_logger (include/dmrg_logger.h:27-99): init before the first sweep,
 * it_log_all after every sweep (sweep number, energy, the sweep's wall seconds,
 * its largest relative discarded weight -- sum of dropped s^2 over sum of all s^2 of
 * a bond's truncation, the weight truncate_impl bounds, btensor_linalg.cpp:658-682 --
 * and the current state), end_log_all once when the driver stops (the last sweep's
 * number, the returned energy, the final state).  The state's handles belong to the
 * library and live for the call only (qtt_bt_clone keeps one).  Any member may be
 * NULL. */
typedef struct {
    void *user;
    void (*init)(void *user, const qtt_dmrg_options *opt);
    void (*it_log_all)(void *user, int64_t step, double energy, double seconds, double truncated_weight, int32_t L,
                       const qtt_bt *mps, int64_t oc);
    void (*end_log_all)(void *user, int64_t step, double energy, int32_t L, const qtt_bt *mps, int64_t oc);
} qtt_dmrg_logger;

/* details::compute_2sitesHamil for one pair (dmrg.h:66; dmrg.cpp:504-515) */
int qtt_compute_2sites_hamil(qtt_bt w_left, qtt_bt w_right, qtt_bt *out);
/* details::hamil2site_times_state (dmrg.h:64; dmrg.cpp:521-531) */
int qtt_hamil2site_times_state(qtt_bt state, qtt_bt hamil, qtt_bt Lenv, qtt_bt Renv, qtt_bt *out);
/* details::one_step_lanczos (dmrg.h:71; dmrg.cpp:585-608) */
int qtt_one_step_lanczos(qtt_bt state, qtt_bt hamil, qtt_bt Lenv, qtt_bt Renv, qtt_bt *psi, double *a0,
                         double *a1, double *b);
/* details::eig2x2Mat (dmrg.h:61; dmrg.cpp:544-572) */
int qtt_eig2x2(double a0, double a1, double b, double *E, double *o, double *n);
/* The all-ones edge environment over leg state_leg of a site tensor and leg mpo_leg of
 * an MPO tensor (generate_env_impl, dmrg.cpp:371-391; edge_shape_prep :335-345): leg 0
 * of the first sites for the left edge, leg 2 of the last sites for the right edge. */
int qtt_trivial_edge(qtt_bt state, int32_t state_leg, qtt_bt mpo, int32_t mpo_leg, qtt_bt *out);
/* compute_left_env / compute_right_env (dmrg.cpp:425-493) */
int qtt_compute_left_env(qtt_bt W, qtt_bt A, qtt_bt Lenv, qtt_bt *out);
int qtt_compute_right_env(qtt_bt W, qtt_bt A, qtt_bt Renv, qtt_bt *out);
/* dmrg(bMPO&, bMPS&, const dmrg_options&, dmrg_logger&) (dmrg.h:39; dmrg.cpp:92-100,219-273).
 * mpo[L], mps[L] (rank-4 and rank-3 btensors); on return mps[] holds NEW handles
 * (the caller destroys the old ones it passed in, and the new ones later);
 * *oc is the orthogonality centre in and out; *E0 the final energy. */
int qtt_dmrg(int32_t L, const qtt_bt *mpo, qtt_bt *mps, int64_t *oc, const qtt_dmrg_options *opt,
             qtt_dmrg_log_fn log_fn, void *log_user, double *E0);
/* The same driver with the full logger interface (dmrg(bMPO&, bMPS&, const
 * dmrg_options&, dmrg_logger&), dmrg.h:39): logger may be NULL. */
int qtt_dmrg_logged(int32_t L, const qtt_bt *mpo, qtt_bt *mps, int64_t *oc, const qtt_dmrg_options *opt,
                    const qtt_dmrg_logger *logger, double *E0);

/* random_bMPS(bond_dim, mpo, constraint, seed) (include/MPT.h:49-53, sources/MPT.cpp:424-462):
 * out[L] receives new rank-3 site tensors whose physical legs are the MPO's leg 1, with
 * total charge constraint[ncomp] (the MPO's group) and bond sectors capped to bond_dim.
 * Entries are N(0, 1) from a counter-based generator keyed by (seed, site, element),
 * each site scaled to unit Frobenius norm; the orthogonality centre is the last site. */
int qtt_random_mps(int32_t L, const qtt_bt *mpo, int64_t bond_dim, const int16_t *constraint, uint64_t seed,
                   qtt_bt *out);

/* <psi|H|psi> and <psi|psi> of an MPS against an MPO, contracted in FP64
 * (contract(bMPS, bMPS, bMPO) and contract(bMPS, bMPS), include/MPT.h; sources/MPT.cpp:211-290). */
int qtt_mps_energy(int32_t L, const qtt_bt *mpo, const qtt_bt *mps, double *energy, double *norm2);

/* ------------------------------------------------------------------ allocation-free SVD
 * No counterpart in QuantiT: an addition for callers that cannot allocate device
 * memory -- a plug-in inside a host application that owns all device memory, a
 * solver under a memory budget fixed at start-up, or a real-time loop that cannot
 * afford cudaMalloc / cudaFree (which can synchronise the whole device).
 * Thin SVD A = U diag(s) V^T of one dense FP64 matrix with the same one-sided
 * Jacobi kernels as the sector SVD, using only a file-scope device array of
 * QTT_SVD_NOALLOC_SCRATCH_BYTES (held by every GPU that loads the library until
 * exit) -- no cudaMalloc / cudaFree and no allocating library routine.
 *   a: m x n row-major (device), u: m x k row-major, s: k, v: n x k row-major
 *   (device outputs), k = min(m, n), m and n <= QTT_SVD_NOALLOC_MAX_DIM; larger
 *   sizes are rejected with QTT_ERR_INVALID_ARGUMENT.  Work is issued on `stream`
 *   (a cudaStream_t, NULL = legacy default stream); the call returns without
 *   waiting for it.
 * The first call on a device (with that device current) looks up the scratch
 * array's device address and sets the kernels' attributes for that device; make
 * that first call before any stream capture.  All calls share the array, which
 * keeps the last call's contents: calls whose work overlaps on the GPU race and
 * corrupt each other's results. */
#define QTT_SVD_NOALLOC_MAX_DIM 256
#define QTT_SVD_NOALLOC_SCRATCH_BYTES (5u * 256u * 256u * 8u + 2048u)
int qtt_svd_dense_noalloc(const double *a, int64_t m, int64_t n, double *u, double *s, double *v, void *stream);

/* ------------------------------------------------------------------ measurement */
/* Per-kernel-class device time (CUDA events on the launching stream) and
 * algorithmic work: kind 0 block GEMM (FLOP), 1 permute (bytes), 2 sector SVD
 * (FLOP, LAPACK-class count 4p^2q + 8pq^2 + 9q^3 per p x q sector), 3 elementwise (bytes),
 * 4 sector pack (bytes), 5 the FP64 stage of the mixed path's sector SVDs (time only; part
 * of kind 2), 6 / 7 the FLOPs the sector SVDs' Jacobi sweeps performed in FP32 / FP64
 * (work only: sweeps x (6 p q^2 + 3 q^3) per p x q sector, plus 8 q^3 + 2 p q^2 for the
 * mixed path's FP64 refinement products; under a truncation the mixed path's FP64 sweeps
 * after the first run on the K kept columns: 6 p K^2 + 3 K^3 each, plus 2 q K^2). */
int qtt_stats_enable(int on);
int qtt_stats_reset(void);
int qtt_stats_get(int kind, double *ms, double *work, int64_t *launches);
/* Number of kernels this library launched since load. */
int64_t qtt_launch_count(void);
/* Jacobi sweeps each sector needed in the most recent decomposition (synchronises);
 * *n receives the sector count, up to cap values are written to out. */
int qtt_last_svd_sweeps(int32_t *out, int32_t cap, int32_t *n);
/* Mixed path only: the FP32 sweeps each sector ran before its FP64 sweeps in the most
 * recent decomposition (*n = 0 after a plain FP64 decomposition; synchronises). */
int qtt_last_svd_fp32_sweeps(int32_t *out, int32_t cap, int32_t *n);

#ifdef __cplusplus
}
#endif
#endif /* QTT_GB300_H */
