/*
 * grafttn.h - C ABI of the GB300 (sm_103a) tree-tensor-network effective-Hamiltonian
 * library (libgrafttn.so).
 *
 * Conventions
 *  - Complex data is interleaved (re, im) double precision (ComplexF64 / complex128).
 *  - A tensor of rank r with leg dims (d0, ..., d{r-1}) is stored row-major: the LAST leg
 *    varies fastest.  A Julia/TensorKit column-major array with legs (l1..lr) is the same
 *    buffer described with its legs (and labels) reversed.
 *  - Leg order inside a tensor follows the reference: TTNS node (children..., phys,
 *    parent), TTNO node (children..., P_out, P_in, parent), environment (ket, op, bra).
 *  - Device buffers are plain CUDA device pointers owned by the caller, unless an entry
 *    point says "host".  All work is ordered on the context's stream.
 *  - Every call returns a gtn_status; gtn_last_error() returns the message of the last
 *    failure on that context.  No exceptions cross the ABI.  Device waits inside kernels
 *    are bounded and surface as GTN_ERR_TIMEOUT.
 *  - A context is used by one host thread at a time (the reference's task-local
 *    WorkspaceMap rule, lib/GraftPlanning/src/Planning/types.jl:503-552).
 */
#ifndef GRAFTTN_H
#define GRAFTTN_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  GTN_OK = 0,
  GTN_ERR_INVALID = 1,        /* bad argument (the reference's ArgumentError) */
  GTN_ERR_SHAPE = 2,          /* leg dimension mismatch (the reference's SpaceMismatch) */
  GTN_ERR_MEMORY = 3,         /* memory admission refused before any launch */
  GTN_ERR_CUDA = 4,           /* CUDA runtime / library error */
  GTN_ERR_TIMEOUT = 5,        /* a bounded device wait gave up */
  GTN_ERR_UNSUPPORTED = 6,    /* feature not available (library missing, arch) */
  GTN_ERR_NOT_CONVERGED = 7   /* Krylov solver hit maxiter (result still returned) */
} gtn_status;

/* Arithmetic of a map application.  The Krylov vectors and all orthogonalisation are
 * FP64 in every mode; the mode selects how the contraction chain is computed. */
typedef enum {
  GTN_PREC_FP64 = 0,       /* complex FP64 throughout (DFMA SIMT kernels) */
  GTN_PREC_BF16X6 = 1,     /* tcgen05: 3 bf16 slices per operand, 6 products, FP32 accum */
  GTN_PREC_BF16X3 = 2,     /* tcgen05: 2 bf16 slices per operand, 3 products, FP32 accum */
  GTN_PREC_FP32 = 3,       /* complex FP32 SIMT kernels (diagnostic mode) */
  GTN_PREC_FP16X3 = 4,     /* tcgen05: 2 fp16 slices per operand (22 bits, power-of-two row
                              scales), 3 products, FP32 accum */
  GTN_PREC_FP64E = 5       /* FP64-grade on the tensor cores: 7 integer base-128 digits per
                              operand (power-of-two row scales), the 28 digit products of
                              level <= 6 summed exactly in FP32 over chunks of 256 k and
                              combined in double-float; about 1e-14 relative (dense maps and
                              one-shot contractions) */
} gtn_precision;

typedef struct gtn_ctx_s* gtn_ctx;
typedef struct gtn_map_s* gtn_map;

/* ---- context --------------------------------------------------------------------- */

/* Create a context on CUDA device `device` with its own non-blocking stream. */
int gtn_ctx_create(int device, gtn_ctx* out);
int gtn_ctx_destroy(gtn_ctx ctx);
/* Use an external cudaStream_t (e.g. the caller's current stream) for all later work. */
int gtn_ctx_set_stream(gtn_ctx ctx, void* stream);
void* gtn_ctx_stream(gtn_ctx ctx);
const char* gtn_last_error(gtn_ctx ctx);
/* Number of library kernels launched on this context so far (launch accounting). */
int64_t gtn_ctx_launch_count(gtn_ctx ctx);
/* Wait for the stream and report (then clear) any device-side error flag. */
int gtn_ctx_sync(gtn_ctx ctx);
/* Precision of the matrix products inside the factorisations of this context (the Gram
 * matrix and the right factor of the truncated SVD's Gram route, gtn_svd_trunc):
 * GTN_PREC_FP64 (default, FP64 SIMT) or GTN_PREC_FP64E (the FP64-grade tensor-core GEMM,
 * about 1e-14 relative to sum |a||b|).  The eigen- and QR decompositions stay cuSOLVER FP64.
 * No counterpart in the reference (its factorisations are LAPACK calls on the host). */
int gtn_ctx_set_linalg_precision(gtn_ctx ctx, int precision);
int gtn_ctx_linalg_precision(gtn_ctx ctx);

/* ---- effective maps: replaces Planning.EffectiveMap / execute / contract_pair ------
 * lib/GraftPlanning/src/Planning/types.jl:410-445 (EffectiveMap callable),
 * lib/GraftPlanning/src/Planning/executor.jl:16-45,99-144 (execute / _execute_workspace),
 * lib/GraftFoundation/src/Backend/Backend.jl:166-222 (contract_pair[!]).
 *
 * A map is an ncon-style label graph over `n_operands` tensors.  Operand 0 is the
 * varying input x; operands 1.. are statics (environments, TTNO tensors, root cap) that
 * are copied / packed into the map at creation, so their buffers may be freed afterwards.
 * labels: positive = contracted pair, -k = output leg k (1-based).  order[] is the
 * pairwise absorption order starting with operand 0 (the reference's env-first
 * preferred_slots order, lib/GraftContractions/src/Contractions/effective.jl:683,971).
 * conj[i] != 0 conjugates operand i (only statics may be conjugated).
 */
int gtn_map_create(gtn_ctx ctx, int n_operands, const int* ranks, const int64_t* dims,
                   const int* labels, const int* conj, const int* order,
                   const void* const* statics, int precision, gtn_map* out);
int gtn_map_destroy(gtn_map map);
/* y = H_eff x on device buffers (c128), in the map's default precision. */
int gtn_map_apply(gtn_map map, const void* x, void* y);
int gtn_map_apply_prec(gtn_map map, int precision, const void* x, void* y);
/* Route this map's FP64 applications (the Rayleigh quotient of gtn_lanczos_min, the
 * residuals of gtn_lanczos_refine, gtn_map_apply_prec with GTN_PREC_FP64) to fp64_map, an
 * FP64 or GTN_PREC_FP64E map of the same shape (e.g. the FP64-grade tensor-core twin of a
 * mixed map); NULL restores the map's own FP64 plan.  fp64_map is not owned: keep it alive
 * while it is set.  No counterpart in the reference (its maps are FP64 only). */
int gtn_map_set_fp64(gtn_map map, gtn_map fp64_map);
/* Same with HOST buffers (one call): host->device copy into a staging buffer the map
 * keeps, apply, device->host copy.  Page-locked buffers (cudaHostAlloc / cudaHostRegister,
 * e.g. a Julia Mem.pin'ed array) make both copies DMA transfers at the link's rate. */
int gtn_map_apply_host(gtn_map map, const void* x_host, void* y_host);
/* Shape/cost facts: elements of x and y, algorithmic FLOPs per apply (complex MAC = 8),
 * number of pair steps, and device workspace bytes held by the map. */
int gtn_map_info(gtn_map map, int64_t* x_elems, int64_t* y_elems, double* flops,
                 int* n_steps, int64_t* bytes);
/* Kernel kinds reported by gtn_map_apply_profiled. */
enum {
  GTN_KERNEL_SMALL = 0,     /* strided small-K contraction (SIMT) */
  GTN_KERNEL_GATHER = 1,    /* permutation of the running tensor into a K-major operand */
  GTN_KERNEL_SPLIT = 2,     /* permutation + bf16 slice split */
  GTN_KERNEL_ZGEMM = 3,     /* complex FP64 SIMT GEMM */
  GTN_KERNEL_CGEMM = 4,     /* complex FP32 SIMT GEMM */
  GTN_KERNEL_TC_GEMM = 5,   /* tcgen05 split-bf16 GEMM */
  GTN_KERNEL_CONVERT = 6,   /* c128 -> c64 input conversion */
  GTN_KERNEL_OUTPUT = 7     /* final permutation into the output leg order */
};
/* One application with CUDA events around every kernel launch (synchronises).  Writes up
 * to `cap` records: duration in ms, kernel kind and algorithmic FLOPs of that launch;
 * *count = number of launches of the application. */
int gtn_map_apply_profiled(gtn_map map, int precision, const void* x, void* y, int cap, double* ms,
                           int* kind, double* flops, int* count);
/* Output leg dims of the map (rank written to *rank, dims to dims[0..rank-1]). */
int gtn_map_out_shape(gtn_map map, int* rank, int64_t* dims);

/* ---- tile shapes of the tensor-core steps ---------------------------------------------
 * The reference chooses how to run a contraction from an analytic cost model
 * (lib/GraftFoundation/src/Backend/Backend.jl:309-368).  Here the tensor-core steps of dense
 * maps choose their tile shape by measurement: the first launch of a problem class (plane
 * count, fp16 or bf16 planes, product count, ceil(log2 M), 2N in steps of 64, ceil(log2
 * k-blocks)) outside stream capture times every candidate tile shape on that problem (one
 * warm-up and two timed launches each, on the caller's stream; this synchronises once) and
 * caches the fastest for the process.  Every candidate computes the same products in the
 * same order per output element, so the choice never changes results.
 * gtn_tc_tuning(mode, clear): mode 0 = fixed ladder, 1 = measured (default), 2 + v = force
 * variant v (0 ps32, 1 ps64, 2 ps128, 3 ps128x2, 4 ps256, 5 pair256 = 256 x 256 tiles on an
 * SM pair, 6 persist128 = persistent 128 x 128, 7 persist256 = persistent 128 x 256) where
 * it is a candidate; mode -1 keeps the mode.  clear != 0 forgets the cached choices.  Returns
 * the previous mode, or -1 for a mode outside -1 .. 9.  Grouped launches (block-sparse steps, batched maps) always run the
 * persistent kernel; in the measured mode their tile width (the widest problem's ladder width
 * or half of it) is measured per problem list the same way.
 * gtn_tc_tune_report writes one text line per cached class (the candidates' times and the
 * choice) into buf (cap bytes, NUL-terminated); *needed = bytes required. */
int gtn_tc_tuning(int mode, int clear);
int gtn_tc_tune_report(char* buf, int64_t cap, int64_t* needed);

/* ---- tensor objects and maps by kind ---------------------------------------------------
 * The reference's drop-in seams hand over TensorMaps and ask for eff_h1 / eff_h2 / eff_h0 /
 * env updates by the node's place in the tree (lib/GraftContractions/src/Contractions/
 * effective.jl:627-797,878-1034; envcache.jl:919-999,1010-1101).  A gtn_tensor is a dense
 * c128 tensor on the context's device (row-major, legs as documented above): library-owned
 * (gtn_tensor_create, then gtn_tensor_upload / gtn_tensor_download from host memory) or a
 * view of the caller's device buffer (gtn_tensor_wrap, e.g. a CuArray; never freed here).
 * gtn_map_create_kind builds the map from a gtn_site_desc and the statics as tensors; the
 * label graph and env-first order are the reference's, the input's dims follow from the
 * statics, and the root cap is supplied by the library.  Statics, in order:
 *   GTN_MAP_H1: W_n, env(w->n) for n's children in slot order, then for n's parent (none at
 *               the root).  Input: A_n (children..., phys, parent).
 *   GTN_MAP_H2: W_n, W_m, env(w->n) for n's children, env(w->m) for m's children except n
 *               in slot order, then for m's parent (none when m is the root).  Input: the
 *               two-site block (n's children..., phys_n, m's other children..., phys_m,
 *               m's parent).
 *   GTN_MAP_H0: env(n->m), env(m->n).  Input: the link matrix C.
 * gtn_env_build writes env(u->v)[ket, op, bra] for GTN_MAP_ENV (n_children, n_is_root
 * describe u; slot = v's child slot of u, or -1 for u's parent) from A_u, W_u and the
 * environments env(w->u) of u's other neighbours (children in slot order, then parent).
 * gtn_site_labels returns the label graph and order of a description (no device needed),
 * always in the row-major leg order. */
typedef struct gtn_tensor_s* gtn_tensor;
enum { GTN_MAP_H1 = 1, GTN_MAP_H2 = 2, GTN_MAP_H0 = 3, GTN_MAP_ENV = 4 };
typedef struct {
  int kind;        /* GTN_MAP_H1 / H2 / H0 / ENV */
  int n_children;  /* children of n (H1, H2) or of u (ENV) */
  int n_is_root;   /* H1: n is the root; ENV: u is the root */
  int m_children;  /* H2: children of m, n's parent */
  int slot;        /* H2: n's child slot in m; ENV: the open neighbour's child slot, -1 = parent */
  int m_is_root;   /* H2: m is the root */
  int col_major;   /* 1: every tensor, the input and the output are column-major arrays with
                      dims given in the reference's leg order (a TensorKit/Julia array's
                      layout, first leg fastest); 0: row-major as everywhere else */
} gtn_site_desc;
int gtn_tensor_create(gtn_ctx ctx, int rank, const int64_t* dims, gtn_tensor* out);
int gtn_tensor_wrap(gtn_ctx ctx, int rank, const int64_t* dims, void* device_data, gtn_tensor* out);
int gtn_tensor_destroy(gtn_tensor t);
void* gtn_tensor_data(gtn_tensor t);
int gtn_tensor_shape(gtn_tensor t, int* rank, int64_t* dims);
int gtn_tensor_upload(gtn_tensor t, const void* host, int64_t elems);
int gtn_tensor_download(gtn_tensor t, void* host, int64_t elems);
int gtn_site_labels(const gtn_site_desc* desc, int cap, int* n_operands, int* ranks, int* labels, int* order);
int gtn_map_create_kind(gtn_ctx ctx, const gtn_site_desc* desc, int n_tensors, const gtn_tensor* tensors,
                        int precision, gtn_map* out);
int gtn_env_build(gtn_ctx ctx, const gtn_site_desc* desc, gtn_tensor A, gtn_tensor W, int n_envs,
                  const gtn_tensor* envs, void* out, int precision);

/* ---- batches of independent maps --------------------------------------------------
 * Replaces the reference's threaded fan-out of many small maps (channel slices,
 * lib/GraftContractions/src/Contractions/effective.jl:26-30,153-165; sibling environment
 * staging, envcache.jl:1164-1304): step s of every map runs in one grouped launch per kernel
 * kind.  All maps must belong to one context; xs/ys are device c128 buffers per map. */
typedef struct gtn_batch_s* gtn_batch;
int gtn_map_apply_batched(int n, const gtn_map* maps, const void* const* xs, void* const* ys,
                          int precision);
/* A fixed batch (maps and buffers); with use_graph != 0 the second gtn_batch_run captures
 * the whole batched application into a CUDA graph and later runs replay it. */
int gtn_batch_create(int n, const gtn_map* maps, const void* const* xs, void* const* ys,
                     int precision, int use_graph, gtn_batch* out);
int gtn_batch_run(gtn_batch batch);
int gtn_batch_destroy(gtn_batch batch);

/* ---- abelian (U(1)) block-sparse maps ----------------------------------------------
 * Replaces TensorKit's per-coupled-charge block GEMMs behind contract_pair for abelian
 * unique-fusion sectors (cost model lib/GraftFoundation/src/Backend/Backend.jl:243-261,
 * 309-368).  A host planner describes every step as GEMM problems (one per coupled charge q:
 * C_q[N][M] = A_q[M][K] * B_q[N][K]^T, B_q a static) and block gathers that assemble A_q
 * from the blocks of the running tensor; the library runs a step as one grouped gather and
 * one grouped GEMM launch.  Buffers: 0 = input x (c128), 1 = output y (c128), 2 and 3 =
 * running buffers (c128 in FP64 mode, c64 otherwise). */
typedef struct {
  int32_t src_buf;     /* 0 = x, 2 or 3 = running buffer */
  int32_t dst_index;   /* step gathers: GEMM problem whose A_q is filled; final gathers: unused */
  int32_t ng_m, ng_k;  /* number of row / column index groups */
  int64_t src_off;     /* block offset in the source buffer (complex elements) */
  int64_t row_off;     /* step: first row in A_q; final: element offset of the block in y */
  int64_t col_off;     /* step: first column in A_q */
  int64_t M, K, Kw;    /* rows, source columns, written columns (zero beyond K) */
  int64_t ld;          /* final: row pitch of the block in y */
  int64_t m_dim[8], m_str[8], k_dim[8], k_str[8];
} gtn_block_gather;
typedef struct {
  int32_t b_index;     /* static B_q [N][K] */
  int32_t c_buf;       /* 2 or 3 */
  int64_t c_off;       /* C_q offset in that buffer (complex elements) */
  int64_t M, N, K;
} gtn_block_gemm;
typedef struct gtn_blockmap_s* gtn_blockmap;
/* statics: nstatics device c128 matrices (copied), static_nk: their (N, K);
 * buffer_elems: complex elements of (x, y, running buffer 2, running buffer 3);
 * flops: algorithmic FLOPs per application (recorded for reporting). */
int gtn_blockmap_create(gtn_ctx ctx, int nsteps, const int* step_ngather, const int* step_ngemm,
                        const gtn_block_gather* gathers, const gtn_block_gemm* gemms, int nfinal,
                        const gtn_block_gather* final_gathers, int nstatics,
                        const void* const* statics, const int64_t* static_nk,
                        const int64_t* buffer_elems, int precision, double flops,
                        gtn_blockmap* out);
int gtn_blockmap_apply(gtn_blockmap map, const void* x, void* y);
/* With use_graph != 0 an application on new (x, y) runs eagerly and is captured into a CUDA
 * graph; later applications on the same (x, y) replay the graph. */
int gtn_blockmap_set_graph(gtn_blockmap map, int use_graph);
int gtn_blockmap_info(gtn_blockmap map, double* flops, int* n_problems, int64_t* bytes);
int gtn_blockmap_destroy(gtn_blockmap map);

/* The eigensolver hook over a block-sparse map (groundstate_eigsolve_backend on abelian
 * TensorMaps, lib/GraftGroundState/src/GroundState/GroundState.jl:25-39): gtn_lanczos_min
 * and gtn_lanczos_refine with the block map as the operator, on the flat block buffer x
 * (every block of the map's input, in its layout).  bm64 (may be NULL when bm is FP64 or
 * neither the FP64 Rayleigh quotient nor refinement is asked for) is the FP64 block map of
 * the same plan: it serves the FP64 applications.  Same arguments and results otherwise. */
int gtn_blockmap_lanczos_min(gtn_blockmap bm, gtn_blockmap bm64, void* x, int krylovdim, double tol,
                             int maxiter, int rq_fp64, double* energy, int* info, double* resid);
int gtn_blockmap_lanczos_refine(gtn_blockmap bm, gtn_blockmap bm64, void* x, int inner_dim, double tol,
                                int max_outer, double* energy, int* info, double* resid);

/* One-shot contraction of a label graph where every operand is given (environment
 * builds, envcache.jl:1010-1101; two-site merge, effective.jl:827-843).  Operand 0 starts
 * the chain; out receives the tensor with legs ordered -1, -2, ... (c128). */
int gtn_contract(gtn_ctx ctx, int n_operands, const int* ranks, const int64_t* dims,
                 const int* labels, const int* conj, const int* order,
                 const void* const* operands, void* out, int precision);

/* Adjoint of one operand of a contraction: the vector-Jacobian product behind an rrule of
 * a map application or an environment update (no counterpart in the reference, which has
 * no AD; gradient rules there would wrap eff_h1/eff_h2 maps, lib/GraftContractions/src/
 * Contractions/effective.jl:709-797, and env updates, envcache.jl:1010-1101).  Takes the
 * label graph and operands of the forward contraction (as gtn_contract / gtn_map_create:
 * operand 0 first, conj flags), a cotangent ybar shaped like the output (legs -1, -2, ...)
 * and writes to out, shaped like operand `slot`, the tensor G with
 *     <G, d op_slot> = <ybar, dy>   (<a, b> = sum conj(a) b)
 * for every perturbation of op_slot as it enters the contraction (after its conj flag):
 * G = contract(ybar, conj(op_i), i != slot).  It runs through the same contraction engine
 * (tcgen05 steps in the mixed precisions).  order (may be NULL) orders the rewritten
 * operand list [ybar, op_i for i != slot]; NULL picks a greedy chain from ybar. */
int gtn_contract_vjp(gtn_ctx ctx, int n_operands, const int* ranks, const int64_t* dims, const int* labels,
                     const int* conj, const int* order, const void* const* operands, int slot, const void* ybar,
                     void* out, int precision);

/* Row-major permutation of a c128 tensor: out has legs (perm[0], perm[1], ...). */
int gtn_permute(gtn_ctx ctx, int rank, const int64_t* dims, const int* perm,
                const void* in, void* out);

/* ---- Krylov solvers: replace the solver hooks ------------------------------------
 * groundstate_eigsolve_backend, lib/GraftGroundState/src/GroundState/GroundState.jl:25-39
 * evolution_exponentiate_backend, lib/GraftEvolution/src/Evolution/Evolution.jl:54-68
 */
/* Lowest eigenpair of the (Hermitian) map by thick-restarted Lanczos on device (about 3/5
 * of the basis kept as Ritz vectors per restart; a local three-term step plus one
 * DGKS-guarded reorthogonalisation pass per iteration).  x (device, c128) holds the start
 * vector on entry and the normalised eigenvector on exit.  With rq_fp64 != 0 the returned
 * energy is the FP64 Rayleigh quotient <x|H x> of the final vector (one FP64 apply).
 * info[0] = restarts, info[1] = matvecs, info[2] = converged flag; resid[0] = residual. */
int gtn_lanczos_min(gtn_map map, void* x, int krylovdim, double tol, int maxiter,
                    int rq_fp64, double* energy, int* info, double* resid);
/* Iterative refinement of an approximate lowest eigenvector (e.g. the result of
 * gtn_lanczos_min on a mixed-precision map) to FP64 accuracy.  Each outer step applies the
 * FP64 plan once to get the residual r = H x - theta x in FP64, builds a Lanczos basis of up
 * to inner_dim vectors from r in the map's own (mixed) precision on the complement of x,
 * and replaces x by the lowest Ritz vector of span(x, basis), whose coupling to x is the
 * exact FP64 |r|.  Stops when |r| <= tol (absolute) or after max_outer corrections.
 * x (device c128): start vector in, normalised refined vector out.  energy = FP64 Rayleigh
 * quotient of the returned x.  info[0] = corrections, info[1] = mixed matvecs, info[2] = FP64
 * matvecs, info[3] = converged; resid = FP64 |r| of the returned x.  The reference has no
 * separate call: its eigsolve hook (lib/GraftGroundState/src/GroundState/GroundState.jl:
 * 25-39) is FP64 throughout, and this call is how the mixed modes meet its accuracy. */
int gtn_lanczos_refine(gtn_map map, void* x, int inner_dim, double tol, int max_outer, double* energy,
                       int* info, double* resid);
/* x <- exp((dz_re + i dz_im) H) x by a Lanczos Krylov exponential with FP64
 * orthogonalisation and sub-stepping to meet tol.  info[0] = substeps, info[1] = matvecs. */
int gtn_expm_apply(gtn_map map, double dz_re, double dz_im, void* x, int krylovdim,
                   double tol, int* info);
/* The same for a map that is not Hermitian (exponentiate with ishermitian = false, as the
 * TDVP sweeps call it for a TTNO without the Hermitian trait, lib/GraftEvolution/src/
 * Evolution/tdvp.jl:204-281): an Arnoldi basis with two FP64 classical Gram-Schmidt
 * passes, exp of the small Hessenberg matrix by scaling and squaring, sub-stepping on the
 * error estimate beta |h(m+1,m)| |e_m^T exp(dz H_m) e_1|.  Same arguments and info. */
int gtn_expm_apply_arnoldi(gtn_map map, double dz_re, double dz_im, void* x, int krylovdim,
                           double tol, int* info);
/* Host utility behind the Arnoldi exponential: E = exp(A) for a dense complex m x m matrix
 * (1 <= m <= 256), row-major with interleaved real and imaginary parts (2 m^2 doubles). */
int gtn_expm_small(int m, const double* A, double* E);

/* ---- factorisations (FP64, cuSOLVER runtime calls) --------------------------------
 * split_svd / TruncationScheme, lib/GraftFoundation/src/Backend/Backend.jl:466-505;
 * left_orth / orth_factor_leg, Backend.jl:602-630.
 */
/* Truncated SVD of the row-major m x n matrix A (device c128).  Keeps
 * r = min(maxdim, #{s > max(atol, rtol*s0)}, discarded-weight rank) >= 1 values.
 * U (m x r, row-major), S (r doubles, HOST), Vh (r x n, row-major) must hold
 * min(m,n) columns/rows of capacity.  *rank = r, *discarded = 2-norm of dropped s.
 * Routes: cuSOLVER gesvd below min(m,n) = 384; above it, subspace iteration on
 * maxdim + max(32, maxdim/2) vectors when four times that fits in min(m,n) and its
 * leading values settle (environment GTN_SVD_SUBSPACE=0 turns it off), else the Gram
 * matrix with Zheevd; rows of Vh are re-orthonormalised by a thin QR after both. */
int gtn_svd_trunc(gtn_ctx ctx, int64_t m, int64_t n, const void* A, int64_t maxdim,
                  double atol, double rtol, double discarded_weight, void* U, double* S,
                  void* Vh, int64_t* rank, double* discarded);
/* Thin QR of the row-major m x n matrix A: Q (m x k), R (k x n), k = min(m, n). */
int gtn_qr(gtn_ctx ctx, int64_t m, int64_t n, const void* A, void* Q, void* R);

/* ---- vector helpers on device c128 buffers (used by the host drivers) ------------- */
int gtn_dot(gtn_ctx ctx, int64_t n, const void* x, const void* y, double* out2);  /* <x,y> */
int gtn_axpby(gtn_ctx ctx, int64_t n, double a_re, double a_im, const void* x,
              double b_re, double b_im, void* y);                                  /* y = a x + b y */
/* Allocation-free batched projections out[j] = <V_j, w> (j < J), complex FP64, for callers
 * that cannot allocate device memory (a host whose own pool owns all HBM, or a loop that
 * cannot take cudaMalloc's device-wide synchronisation).  No counterpart in the reference.
 * Needs no context: runs on `stream` (a cudaStream_t, NULL = legacy default) of the current
 * device.  V holds J vectors of n elements, `ldv` elements apart (ldv >= n when J > 1);
 * w has n elements; out (device) receives J values.  Limits: 1 <= J <= 64; partial sums
 * live in a library-owned 512 KiB __device__ array shared by all calls on a device, so
 * calls that overlap on the GPU race (order them on one stream).  The first call on each
 * device resolves that array's address (cached until exit; it does not survive
 * cudaDeviceReset); make it before any stream capture.  Returns GTN_ERR_INVALID for J
 * outside 1..64 or bad pointers / strides, and GTN_ERR_CUDA without launching when an
 * earlier CUDA error is pending on the calling thread (left for the caller to read);
 * never allocates. */
int gtn_multidot_noalloc(void* stream, int64_t n, int J, const void* V, int64_t ldv, const void* w,
                         void* out);

/* One leg of a row-major c128 tensor restricted to an index list (host int64, each below
 * dims[leg]): out has the same legs with dims[leg] replaced by nsel,
 * out[..., j, ...] = in[..., idx[j], ...].  This is the operator-channel restriction of a
 * channel-sliced map's statics (the TTNO leg and the matching environment leg;
 * lib/GraftContractions/src/Contractions/effective.jl:445-520), done on the device. */
int gtn_restrict_leg(gtn_ctx ctx, int rank, const int64_t* dims, int leg, int64_t nsel, const int64_t* idx,
                     const void* in, void* out);

/* x[i] = re + i im for i < n (device c128): zero-filled work buffers of the host drivers. */
int gtn_fill(gtn_ctx ctx, int64_t n, double re, double im, void* x);

/* Strided 2-D copy of c128 data: dst[i*dst_ld + j] = src[i*src_ld + j] for i < rows, j < cols
 * (column concatenation of factors, e.g. the expanded isometry [Q E] of a bond expansion). */
int gtn_copy2d(gtn_ctx ctx, int64_t rows, int64_t cols, const void* src, int64_t src_ld, void* dst,
               int64_t dst_ld);

/* In-place diagonal scaling of a row-major rows x cols c128 matrix by real HOST factors:
 * side 0 scales column j by d[j] (U * diag(S)), side 1 scales row i by d[i] (diag(S) * Vh). */
int gtn_diag_scale(gtn_ctx ctx, int64_t rows, int64_t cols, const double* d_host, int side, void* A);

/* Failure-path self-test: one device thread waits on an mbarrier that nothing arrives at,
 * with the same bounded-wait code as the tensor-core kernels but a limit of `timeout_us`
 * microseconds (1..2000000); it then records a timeout in the context's error flag and
 * returns.  The next gtn_ctx_sync reports GTN_ERR_TIMEOUT and clears the flag; the context
 * stays usable.  No counterpart in the reference (its device-free code has no waits). */
int gtn_selftest_wait(gtn_ctx ctx, int64_t timeout_us);

#ifdef __cplusplus
}
#endif
#endif /* GRAFTTN_H */
