/* C ABI of the GB300 direct-SCF J/K engine (libgb300jk.so).
 *
 * Plain pointers and sizes only.  Device pointers are caller-owned CUDA
 * device memory of the current device; the library owns a workspace inside
 * each optimizer (pair data, screening tables, work lists, scratch
 * accumulators).  All entry points return 0 on success or a negative error
 * code; jk_last_error() gives a message for the last failure on the calling
 * thread.  Work is enqueued on the caller's stream; calls on one optimizer
 * must not overlap.
 *
 * Which reference interface each entry point replaces:
 *   jk_opt_create   gpu4pyscf/scf/jk.py:407-442 (_VHFOpt.__init__/build) and
 *                   jk.py:984-1120 (_cache_q_cond_and_non0pairs), including
 *                   int2e_qcond_estimator (lib/gvhf-rys/nr_sr_estimator.cu:416)
 *   jk_build        RYS_build_jk (lib/gvhf-rys/rys_contract_jk.cu:344-350),
 *                   RYS_build_k (rys_contract_k.cu:605-612) and the class loop
 *                   of _VHFOpt.get_jk (jk.py:492-641), for the sorted basis
 *   jk_opt_destroy  release of the GPU caches held by _VHFOpt (jk.py:418-421)
 *   jk_last_error   the stderr message + int status of RYS_build_jk
 *                   (rys_contract_jk.cu:442-452)
 *   jk_energy_grad  RYS_per_atom_jk_ip1 (lib/gvhf-rys/rys_contract_jk_ip1.cu:
 *                   1747-1797) and the class loop of _jk_energy_per_atom
 *                   (grad/rhf.py:60-171)
 * The remaining entry points (batched builds, range separation, the
 * allocation-free build, autotuning, deterministic accumulation) say at
 * their declaration what they replace or that the reference has none.
 */
#ifndef GB300JK_H
#define GB300JK_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct jk_opt jk_opt;

/* Precision modes of jk_build */
#define JK_PREC_FP64 0   /* every quartet in FP64 */
#define JK_PREC_MIXED 1  /* quartets whose bound < split_thresh in FP32, FP64 accumulation;
                            large-T Rys roots of those quartets in FP64 */
#define JK_PREC_MIXED_FP32ROOTS 2  /* as JK_PREC_MIXED, large-T roots in FP32 as well */

/* Error codes */
#define JK_OK 0
#define JK_ERR_ARG -1
#define JK_ERR_CUDA -2
#define JK_ERR_LMAX -3
#define JK_ERR_ALLOC -4
#define JK_ERR_OVERFLOW -5

typedef struct {
    int64_t quartets_fp64;      /* shell quartets computed in FP64 (after screening) */
    int64_t quartets_fp32;      /* shell quartets computed in FP32 */
    int64_t prim_quartets_fp64; /* primitive quartets behind quartets_fp64 */
    int64_t prim_quartets_fp32;
    int64_t flops_fp64;         /* algorithmic FLOPs of the FP64 quartets (model in the docs) */
    int64_t flops_fp32;
    int32_t kernel_launches;
    int32_t n_classes;
} jk_stats;

/* Build the screening optimizer for a basis already in sorted order
 * (shells ordered by angular momentum, one contraction per shell,
 * coefficients including the radial normalisation, Cartesian functions).
 * atm[natm*6], bas[nbas*8], env[nenv] use the libcint layout.
 * tol: direct_scf_tol (quartets with bound below it are skipped).
 * flags: reserved, pass 0. */
int jk_opt_create(const int32_t *atm, int natm, const int32_t *bas, int nbas,
                  const double *env, int nenv, double tol, int flags, jk_opt **out);

/* Optimizer for a batch of molecules sharing every class launch (no
 * counterpart in the reference, which loops over molecules in Python).
 * The shells of all molecules, each molecule's sorted Cartesian basis, are
 * merged and sorted by angular momentum; shell_mol[i] is the molecule of
 * shell i, shell_ao[i] its first AO within that molecule and mol_nao[m] the
 * AOs of molecule m.  Shell pairs and quartets never mix molecules.
 * Densities and J/K of a batch are packed: density idm holds, for each
 * molecule in order, its nao_m x nao_m block (jk_opt_ntot() elements per
 * density). */
int jk_opt_create_batch(const int32_t *atm, int natm, const int32_t *bas, int nbas,
                        const double *env, int nenv, const int32_t *shell_mol,
                        const int32_t *shell_ao, int nmol, const int32_t *mol_nao,
                        double tol, int flags, jk_opt **out);

void jk_opt_destroy(jk_opt *opt);

/* Densities each molecule of a batch carries (host array [nmol]; NULL
 * clears): later builds skip the digestion of density slots beyond a
 * molecule's count, so molecules with fewer densities than the batch's
 * n_dm cost no more than their own.  Those slots must hold zeros. */
int jk_opt_set_mol_ndm(jk_opt *opt, const int32_t *ndm);

/* Elements per packed density of the optimizer (nao^2 for one molecule). */
long long jk_opt_ntot(const jk_opt *opt);

/* Number of Cartesian AOs of the sorted basis. */
int jk_opt_nao(const jk_opt *opt);

/* Number of atoms of the basis the optimizer was created with. */
int jk_opt_natm(const jk_opt *opt);

/* Number of significant shell pairs kept after Schwarz screening. */
int jk_opt_npairs(const jk_opt *opt);

/* Per-shell-pair Schwarz factors sqrt(max|(ij|ij)|) as computed on the GPU,
 * written to host array q[nbas*nbas] (symmetric; 0 for pruned pairs). */
int jk_opt_get_qcond(const jk_opt *opt, double *q);

/* J/K for n_dm densities in the sorted Cartesian basis.
 * dm: device [n_dm][nao][nao] float64, C order.
 * hermi: 0 general, 1 symmetric, 2 antisymmetric (vj set to zero).
 * vj, vk: device [n_dm][nao][nao] float64 outputs (either may be NULL when
 *         with_j / with_k is 0).
 * precision: JK_PREC_FP64, JK_PREC_MIXED or JK_PREC_MIXED_FP32ROOTS with
 *            split_thresh the bound below which a quartet is evaluated in FP32.
 * stream: cudaStream_t of the caller (NULL = legacy default stream).
 * stats: optional host output. */
int jk_build(jk_opt *opt, const double *dm, int n_dm, int nao, int hermi,
             int with_j, int with_k, int precision, double split_thresh,
             double *vj, double *vk, void *stream, jk_stats *stats);

/* J/K of a batch optimizer: dm, vj, vk are packed [n_dm][jk_opt_ntot()]
 * (one block per molecule, see jk_opt_create_batch); otherwise as jk_build.
 * For one molecule it equals jk_build. */
int jk_build_batch(jk_opt *opt, const double *dm, int n_dm, int hermi,
                   int with_j, int with_k, int precision, double split_thresh,
                   double *vj, double *vk, void *stream, jk_stats *stats);

/* J/K with the range-separated operator
 *     lr_factor * erf(|omega| r)/r + sr_factor * erfc(|omega| r)/r
 * for both J and K; otherwise as jk_build.  Replaces the omega / lr_factor /
 * sr_factor arguments of RYS_build_k (gpu4pyscf/lib/gvhf-rys/
 * rys_contract_k.cu:605-612) and the omega that RYS_build_jk reads from the
 * basis environment (env[8], libcint's PTR_RANGE_OMEGA), with the factor
 * convention of gpu4pyscf/scf/jk.py:1122-1168 resolved by the caller:
 * omega > 0 with (1, 0) is erf(omega r)/r, (0, 1) is erfc(|omega| r)/r.
 * omega = 0 requires lr_factor == sr_factor (the Coulomb operator scaled).
 * The short-range part is evaluated as full range minus long range (one
 * extra pass of every class kernel); screening uses the full-range Schwarz
 * factors, which bound both parts. */
int jk_build_rsh(jk_opt *opt, const double *dm, int n_dm, int nao, int hermi,
                 int with_j, int with_k, double omega, double lr_factor, double sr_factor,
                 int precision, double split_thresh, double *vj, double *vk,
                 void *stream, jk_stats *stats);

/* Nuclear gradient of the J/K energy; replaces RYS_per_atom_jk_ip1
 * (gpu4pyscf/lib/gvhf-rys/rys_contract_jk_ip1.cu:1747-1797) as called by
 * _jk_energy_per_atom (gpu4pyscf/grad/rhf.py:60-171).
 * ejk[A][x] = dE/dR_A,x of
 *     E = j_factor/2 sum (ij|kl) D_ji D_lk - k_factor/4 sum (ij|kl) D_jk D_li
 * at fixed densities, for a symmetric or antisymmetric density (n_dm = 1,
 * an RHF density; the K weight uses D_jk D_li + D_jl D_ki) or a pair of
 * spin densities (n_dm = 2: J of their sum, K of each, k_factor not
 * halved), the reference's weights for both.
 * dm: device [n_dm][nao][nao] float64 in the sorted Cartesian basis of a
 *     single-molecule optimizer.
 * omega, lr_factor, sr_factor: the operator as in jk_build_rsh (0, 1, 1 for
 *     the Coulomb operator).
 * ejk: device [jk_opt_natm()][3] float64 output, overwritten.
 * Screening: q_ij q_kl times the largest density product of the quartet's
 * weight against the optimizer's tolerance.  Shells up to f
 * (JK_ERR_LMAX above).  Asynchronous on stream unless stats (optional host
 * output: quartets and primitive quartets evaluated, in the FP64 fields) is
 * given, which synchronises. */
int jk_energy_grad(jk_opt *opt, const double *dm, int n_dm, int nao, double j_factor,
                   double k_factor, double omega, double lr_factor, double sr_factor,
                   double *ejk, void *stream, jk_stats *stats);

/* Products with the sparse map C between the user basis and the sorted
 * basis, given as compressed rows S = (ptr[rows+1], idx, val) in device
 * memory; replaces the dense C / C^T products of SortedGTO.apply_C_mat_CT
 * and apply_CT_mat_C (gpu4pyscf/gto/mole.py:906-938).
 *   side 0 (right): out[i][r][m] = sum_p in[i][r][idx[p]] val[p] over row m
 *                   of S (S has M rows, idx < K); in [n][R][K]
 *   side 1 (left):  out[i][r][m] = sum_p val[p] in[i][idx[p]][m] over row r
 *                   of S (S has R rows, idx < K); in [n][K][M]
 * out [n][R][M].  C D C^T is right then left with S = C (rows: sorted AOs);
 * C^T V C right then left with S = C^T.  The index arrays are the
 * caller's to keep in range.  Asynchronous on stream. */
int jk_sparse_mm(int side, const int *ptr, const int *idx, const double *val, int n, int R, int K, int M,
                 const double *in, double *out, void *stream);

/* Autotuner (no counterpart in the reference, whose launch schemes are
 * fixed per class).  jk_opt_tune times, for every angular class (and
 * precision) the optimizer launches, each kernel family the class has
 * (register-resident, block-cooperative) with grids of 1, 2, 4 and 8 blocks
 * per SM on the given densities (best of reps launches) and keeps the
 * fastest for later builds.  dm as in jk_build_batch.  Synchronises.
 * jk_opt_set_variant / jk_opt_get_variant set or read the choice of class
 * q (0 .. jk_n_quartet_classes()-1) and precision prec (0 FP64, 1 FP32):
 * alt 0 default family, 1 the alternative; grid_per_sm 0 = default. */
int jk_opt_tune(jk_opt *opt, const double *dm, int n_dm, int hermi, int precision,
                double split_thresh, void *stream, int reps);
int jk_opt_set_variant(jk_opt *opt, int q, int prec, int alt, int grid_per_sm);
int jk_opt_get_variant(const jk_opt *opt, int q, int prec, int *alt, int *grid_per_sm);

/* Deterministic accumulation (no counterpart in the reference, whose FP64
 * atomics make J/K depend on the order the GPU adds them in).  When enabled,
 * later jk_build / jk_build_batch / jk_build_rsh calls of this optimizer add
 * every contribution as two 64-bit fixed-point integers per element
 * (multiples of 2^-24 and of 2^-56), whose sums do not depend on the order
 * of the additions: J and K are bitwise reproducible from run to run, within
 * 2^-57 per contribution of the default FP64 accumulation.  Costs an extra
 * 16 bytes per J/K element of workspace and a few FP64 instructions per
 * atomic.  jk_build_noalloc does not use it. */
int jk_opt_set_deterministic(jk_opt *opt, int enable);

const char *jk_last_error(void);

/* One-electron integrals over the raw Cartesian functions of a sorted basis
 * (same layout rules as jk_opt_create): overlap S, kinetic T and nuclear
 * attraction V (point nuclei of all atoms), device outputs [nao][nao].
 * Replaces the int1e_ovlp / int1e_kin / int1e_nuc integrals that gpu4pyscf's
 * SCF driver takes for get_ovlp / get_hcore (gpu4pyscf/scf/hf.py:138-155).
 * Synchronises the stream before returning. */
int jk_int1e(const int32_t *atm, int natm, const int32_t *bas, int nbas,
             const double *env, int nenv, double *S, double *T, double *V, void *stream);
const char *jk_int1e_last_error(void);

/* Diagnostics (no counterpart in the reference).
 * jk_opt_time_classes: when enabled, every class launch of later jk_build
 * calls is bracketed by CUDA events on the build's stream.
 * jk_opt_class_times: after a build, per quartet class q (and precision p,
 * index 2*q+p) the kernel time in ms and the algorithmic FLOPs counted in the
 * last build made with stats; li/lj/lk/ll receive the angular momenta.
 * The caller's arrays hold jk_n_quartet_classes()*2 entries (li..ll: *1). */
int jk_n_quartet_classes(void);
int jk_opt_time_classes(jk_opt *opt, int enable);
int jk_opt_class_times(jk_opt *opt, double *ms, int64_t *flops, int64_t *quartets,
                       int32_t *li, int32_t *lj, int32_t *lk, int32_t *ll);

/* FMA-chain throughput probe: runs iters dependent-chain FMAs (8 chains per
 * thread) on blocks*256 threads in FP64 (fp32=0) or FP32 (fp32=1) and writes
 * a checksum to out[0] (device memory).  Used to measure the FP64/FP32 pipe
 * peak that the roofline of the J/K kernels is reported against. */
int jk_probe_fma(double *out, int blocks, int iters, int fp32, void *stream);

/* Allocation-free J/K build.  No counterpart in the reference: gpu4pyscf
 * always allocates its buffers with CuPy.
 *
 * For callers that may not allocate device memory once they are running:
 * processes held to a fixed device-memory budget after start-up, and host
 * applications whose own framework owns every device allocation and forbids
 * a library from calling cudaMalloc.  jk_build grows a per-optimizer
 * workspace on demand; this entry point calls no cudaMalloc, cudaFree or
 * allocating library routine.  Same arguments and results as jk_build
 * (without stats), including the optimizer's launch variants and the
 * precision modes.  Every per-call buffer comes from one fixed device array of
 * jk_noalloc_scratch_bytes() bytes (32 MiB) that every GPU loading this
 * library holds until the process exits; a call needs about
 * 8*nao^2*(2*n_dm + 2*n_dmk) bytes (n_dmk = 2*n_dm for hermi=0, else n_dm),
 * plus 4*nao^2*(n_dm + n_dmk) in mixed precision and 4*nbas^2 for the
 * screening table, and is rejected with JK_ERR_OVERFLOW above the limit.
 * The optimizer must come from jk_opt_create beforehand (that call does
 * allocate).  The first call on a device also does a one-time set-up: it
 * looks up the array's device address (cudaGetSymbolAddress) with that
 * device current; make that first call before any stream capture.  Every
 * call clears the parts of the array that must start at zero, and the array
 * keeps the last call's contents otherwise.  All calls share the one array,
 * so calls that overlap on the GPU (other streams, other optimizers, other
 * host threads) race: serialise them. */
int jk_noalloc_scratch_bytes(void);
int jk_build_noalloc(jk_opt *opt, const double *dm, int n_dm, int nao, int hermi,
                     int with_j, int with_k, int precision, double split_thresh,
                     double *vj, double *vk, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* GB300JK_H */
