/*
 * tnfa.h -- flat C ABI of libtnfa, the GB300 (sm_103a) engine for quantics
 * tree tensor network functions.
 *
 * A "network" (tnfa_net) is a tree -- or a forest -- of dense tensors held in
 * device memory.  Each vertex carries zero or more site legs (one per quantics
 * digit; an operator carries out/in pairs fused into one leg of dim base^2),
 * one bond to its parent (dimension 1 for a root) and one bond per child.
 *
 * Canonical tensor layout (host <-> device): per vertex a row-major array with
 * axes [site legs in declaration order..., parent bond, child bonds in
 * ascending vertex order]; vertices concatenated in vertex order.  Vertices are
 * topologically ordered: parent[v] < v, parent[root] = -1.
 *
 * Every entry point returns a tnfa_status.  No exception crosses the ABI.  The
 * caller owns every host buffer; the library owns tnfa_ctx / tnfa_net objects
 * and frees them in the matching *_destroy call.  Calls on one context are
 * ordered on that context's stream; a context must be used by one host thread
 * at a time.
 *
 * Each declaration names the reference function it replaces (paths are within
 * the ITensorNumericalAnalysis.jl project).
 */
#ifndef TNFA_H
#define TNFA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

typedef enum {
  TNFA_OK = 0,
  TNFA_ERR_INVALID_ARGUMENT = 1, /* null pointer, bad enum, size mismatch        */
  TNFA_ERR_CUDA = 2,             /* a CUDA runtime call failed                    */
  TNFA_ERR_OUT_OF_MEMORY = 3,    /* device allocation failed                      */
  TNFA_ERR_TOPOLOGY = 4,         /* parent[] not a topologically ordered forest   */
  TNFA_ERR_SHAPE = 5,            /* bond / site dimensions of operands disagree   */
  TNFA_ERR_DTYPE = 6,            /* element type not supported by this entry      */
  TNFA_ERR_NOT_CONVERGED = 7,    /* iterative factorisation / solver hit its cap  */
  TNFA_ERR_TIMEOUT = 8,          /* a device-side wait ran out of its budget      */
  TNFA_ERR_DOMAIN = 9,           /* a coordinate is negative or not finite        */
  TNFA_ERR_UNSUPPORTED = 10      /* valid request the library does not implement  */
} tnfa_status;

typedef enum { TNFA_F64 = 0, TNFA_F32 = 1, TNFA_C128 = 2 } tnfa_dtype;

typedef enum { TNFA_MEM_HOST = 0, TNFA_MEM_DEVICE = 1 } tnfa_memory;

/* Arithmetic used by tnfa_evaluate. */
typedef enum {
  TNFA_PREC_F64 = 0,       /* plain FP64 on the CUDA cores                                 */
  TNFA_PREC_F32 = 1,       /* FP32 on the CUDA cores                                       */
  TNFA_PREC_MIXED = 2,     /* FP64 messages; two-child vertices (bonds 64/128) as exact
                              products of 8-bit integer slices on the tcgen05 tensor cores
                              (26 BF16 passes, FP32 accumulation exact), FP64-class result.
                              In truncation: FP32-preconditioned Jacobi with a
                              double-float (FP32 pair) polish.                             */
  TNFA_PREC_MIXED_FAST = 3 /* FP32 messages, tcgen05 split-BF16 (hi/lo, 3 passes) products:
                              about 1e-5 relative (norm-wise) on random bond-128 trees     */
} tnfa_precision;

/* Leg kinds (tnfa_topology.leg_kind). */
typedef enum {
  TNFA_LEG_REAL = 0,     /* digit of the real part of a variable            */
  TNFA_LEG_IMAG = 1,     /* digit of the imaginary part (complex index map)  */
  TNFA_LEG_OPERATOR = 2  /* fused (out, in) leg of an operator, dim base^2   */
} tnfa_leg_kind;

/* Output encodings of tnfa_evaluate. */
typedef enum {
  TNFA_OUT_F64 = 0,        /* double per point (real networks)                        */
  TNFA_OUT_F32 = 1,        /* float per point (may under/overflow)                    */
  TNFA_OUT_F32_SCALED = 2, /* float mantissa + int32 base-2 exponent per point:
                              value = out_f32[p] * 2^out_i32[p]; the i32 array follows
                              the f32 array in the same buffer (8 bytes per point)    */
  TNFA_OUT_C128 = 3        /* (re, im) double pair per point (complex networks)      */
} tnfa_out;

typedef struct tnfa_ctx tnfa_ctx;
typedef struct tnfa_net tnfa_net;

typedef struct {
  int32_t n_vertices;
  const int32_t* parent;    /* [n_vertices]  parent vertex, -1 for a root; parent[v] < v   */
  const int32_t* link_dim;  /* [n_vertices]  dim of bond (v, parent[v]); must be 1 at roots */
  const int32_t* n_legs;    /* [n_vertices]  number of site legs at v (may be 0)            */
  const int32_t* leg_dim;   /* [sum n_legs]  leg dimension (base, or base^2 for operators)  */
  const int32_t* leg_var;   /* [sum n_legs]  1-based continuous variable of the leg         */
  const int32_t* leg_digit; /* [sum n_legs]  1-based digit, 1 = most significant            */
  const int32_t* leg_kind;  /* [sum n_legs]  tnfa_leg_kind                                  */
} tnfa_topology;

typedef struct {
  double cutoff;     /* relative discarded weight: sum(dropped s^2)/sum(s^2) <= cutoff */
  int32_t maxdim;    /* 0 = unbounded                                                  */
  int32_t mindim;    /* >= 1                                                           */
  int32_t normalize; /* nonzero: rescale the result to unit 2-norm                     */
  int32_t precision; /* tnfa_precision of the contractions                             */
} tnfa_trunc_params;

/* ---- context ------------------------------------------------------------ */

/* Bind to `device` and order all work on `stream` (a cudaStream_t; NULL = the
 * library creates its own stream). */
int tnfa_ctx_create(int device, void* stream, tnfa_ctx** out);
int tnfa_ctx_destroy(tnfa_ctx* ctx);
int tnfa_ctx_synchronize(tnfa_ctx* ctx);
/* Message of the last failing call on this context ("" if none). */
const char* tnfa_last_error_string(const tnfa_ctx* ctx);
/* Library version string, e.g. "tnfa 0.1.0 sm_103a". */
const char* tnfa_version(void);

/* Kernel accounting (no reference counterpart; used by benchmarks).  Every
 * kernel launch is counted per family ("contract_tc", "contract_simt",
 * "digitize", ...) together with its algorithmic flops and bytes; with timing
 * enabled each launch is also bracketed by CUDA events on the context stream.
 * tnfa_ctx_kernel_stats synchronises the stream and returns up to `max`
 * families: names (32 bytes each, NUL-terminated), launches, summed duration
 * in ms (0 when timing was off), flops and bytes.  reset != 0 clears the
 * counters afterwards. */
int tnfa_ctx_set_timing(tnfa_ctx* ctx, int enable);

/* Autotuning of interchangeable launch variants (the SIMT contraction's tile
 * shape, the tensor-core evaluation's formulation).  The first call that
 * meets a shape whose algorithmic work reaches min_work flops times every
 * variant once on the context's stream and keeps the fastest for that shape;
 * later calls reuse it.  enable: 1 on, 0 off (rule-based choice), -1 keep
 * (the default comes from the environment variable TNFA_AUTOTUNE, on unless
 * it is "0"); min_work < 0 keeps the threshold (default 2e9); forget != 0
 * drops the kept choices.  No counterpart in the reference (its contractions
 * are BLAS calls). */
int tnfa_ctx_set_autotune(tnfa_ctx* ctx, int enable, double min_work, int forget);
/* The kept choices, one line each: "<shape key> <variant> <ms per variant...>".
 * Writes at most size bytes (NUL-terminated) and the full size into *needed. */
int tnfa_ctx_tuning_report(tnfa_ctx* ctx, char* buf, int64_t size, int64_t* needed);
int tnfa_ctx_kernel_stats(tnfa_ctx* ctx, int32_t max, char* names, int64_t* launches, double* ms,
                          double* flops, double* bytes, int32_t* n_families, int reset);

/* Wait budget of the tensor-core pipelines: every mbarrier wait in a tcgen05
 * kernel gives up after `polls` try_wait polls (0 keeps the current budget;
 * the default is 2^26), the kernel stops, releases its tensor memory and the
 * call returns TNFA_ERR_TIMEOUT.  drop_arrive != 0 is a test switch: the
 * sliced tensor-core evaluation then withholds the arrive that releases its
 * MMA issuer, so that a wait runs out (with a small budget) and the timeout
 * path can be exercised; 0 restores normal operation.  No counterpart in the
 * reference (it has no device pipelines). */
int tnfa_ctx_set_wait_budget(tnfa_ctx* ctx, uint32_t polls, int drop_arrive);

/* Fault injection for tests of the error paths.  fail_alloc_after >= 0: the
 * next fail_alloc_after device allocations of this context succeed and the
 * one after fails as if the device were out of memory (the call returns
 * TNFA_ERR_OUT_OF_MEMORY and releases what it held); -1 turns it off.
 * jacobi_sweep_cap > 0 caps every one-sided Jacobi SVD at that many sweeps,
 * so that a truncation that needs more returns TNFA_ERR_NOT_CONVERGED; 0
 * restores the built-in caps.  No counterpart in the reference. */
int tnfa_ctx_inject_faults(tnfa_ctx* ctx, int64_t fail_alloc_after, int32_t jacobi_sweep_cap);

/* ---- networks ----------------------------------------------------------- */

/* Build a network from the canonical layout.  Replaces the construction of an
 * ITensorNetworkFunction (src/itensornetworkfunction.jl:18-22) paired with its
 * IndsNetworkMap (src/indsnetworkmap.jl:9-13, src/IndexMaps/realindexmap.jl:6-9,
 * src/IndexMaps/complexindexmap.jl:6-10).  `tensors` is n_elements scalars of
 * `dtype` in host or device memory. */
int tnfa_net_create(tnfa_ctx* ctx, const tnfa_topology* topo, int dtype, const void* tensors,
                    int memory, tnfa_net** out);
int tnfa_net_destroy(tnfa_net* net);
/* Shape query: n_vertices, dtype, total element count; link_dim_out (may be
 * NULL) receives the current bond dimensions (they change under truncation). */
int tnfa_net_info(const tnfa_net* net, int32_t* n_vertices, int32_t* dtype, int64_t* n_elements,
                  int32_t* link_dim_out);
/* Copy the tensors back in canonical layout (n_elements scalars). */
int tnfa_net_download(tnfa_ctx* ctx, const tnfa_net* net, void* tensors, int memory);
/* Deep copy (src/itensornetworkfunction.jl:33-35 Base.copy). */
int tnfa_net_copy(tnfa_ctx* ctx, const tnfa_net* net, tnfa_net** out);
/* Multiply the tensor of `vertex` by the scalar (re, im); im must be 0 for
 * real networks.  Used by the constructors' `c` factors
 * (src/elementary_functions.jl:50,98,102) and scalar * function. */
int tnfa_net_scale(tnfa_ctx* ctx, tnfa_net* net, int32_t vertex, double re, double im);

/* ---- evaluation (hot path) ---------------------------------------------- */

/* Batched point evaluation f(x_p), p < n_points.  Replaces evaluate
 * (src/itensornetworkfunction.jl:96-112), i.e. calculate_ind_values
 * (src/IndexMaps/realindexmap.jl:67-76, src/IndexMaps/abstractindexmap.jl:121-138;
 * complex maps src/IndexMaps/complexindexmap.jl:116-132), project
 * (src/itensornetworkfunction.jl:84-94) and the tree contraction scalar(tn; alg="bp").
 * X: n_points x n_cols row-major doubles, column j holding variable dims[j]
 * (1-based); for networks with TNFA_LEG_IMAG legs n_cols = 2*n_dims with
 * (re, im) per variable.  Every variable that has a leg must be listed.
 * out: per `out_kind` (tnfa_out).  A negative / non-finite coordinate gives
 * TNFA_ERR_DOMAIN (the reference's digit loop never terminates for those). */
int tnfa_evaluate(tnfa_ctx* ctx, const tnfa_net* net, const double* X, int64_t n_points,
                  int32_t n_dims, const int32_t* dims, int x_memory, void* out, int out_kind,
                  int out_memory, int precision);

/* Batched evaluation for callers that cannot allocate device memory during
 * the call -- for example code whose GPU memory is wholly owned by another
 * runtime's caching allocator (where cudaMalloc would fail or implicitly
 * synchronise the device), or latency-bound serving loops that must not block
 * on the allocator.  No counterpart in the reference (its evaluate allocates
 * freely on the host).  It computes what tnfa_evaluate computes, with every
 * scratch buffer taken from one fixed 32 MiB device array compiled into the
 * library (each GPU that loads the library holds it until exit) and no
 * cudaMalloc / cudaFree.  X (n_points x n_cols doubles) and out must be device
 * pointers; precision must match the network's type (TNFA_PREC_F64 on FP64 or
 * complex networks, TNFA_PREC_F32 on FP32 networks).  A request whose scratch
 * does not fit is rejected with TNFA_ERR_INVALID_ARGUMENT, naming the number of
 * points that fit.  The first call on a device looks up the array's device
 * address; make that call before any stream capture.  All calls share the one
 * array, so calls that overlap on the GPU (other streams, other host threads)
 * race: serialise them. */
int tnfa_evaluate_noalloc(tnfa_ctx* ctx, const tnfa_net* net, const double* X, int64_t n_points,
                          int32_t n_dims, const int32_t* dims, void* out, int out_kind,
                          int precision);

/* Captured evaluation for repeated calls on fixed device buffers: the
 * kernel sequence of tnfa_evaluate_noalloc for n_points points read from X
 * and written to out (both device pointers, fixed for the plan's life) is run
 * once eagerly (validating the inputs; out holds its result), then captured
 * into a CUDA graph over scratch the plan owns.  tnfa_eval_plan_launch
 * enqueues one graph launch on the context's stream: it evaluates whatever X
 * holds at that point in stream order and returns without waiting.
 * tnfa_eval_plan_check waits for the stream and reports TNFA_ERR_DOMAIN if
 * the last launch met a negative or non-finite coordinate.  The plan reads
 * the network's tensors where they were at creation: the network must
 * outlive the plan, and in-place changes to its values are seen by later
 * launches.  No counterpart in the reference (one evaluate call per point,
 * itensornetworkfunction.jl:96-112); it serves latency-bound loops
 * (optimisers, samplers) that evaluate the same number of points many times.
 * Precision as for tnfa_evaluate_noalloc.  Do not call from inside another
 * stream capture. */
typedef struct tnfa_eval_plan tnfa_eval_plan;
int tnfa_eval_plan_create(tnfa_ctx* ctx, const tnfa_net* net, const double* X, int64_t n_points,
                          int32_t n_dims, const int32_t* dims, void* out, int out_kind,
                          int precision, tnfa_eval_plan** plan);
int tnfa_eval_plan_launch(tnfa_ctx* ctx, tnfa_eval_plan* plan);
int tnfa_eval_plan_check(tnfa_ctx* ctx, tnfa_eval_plan* plan);
int tnfa_eval_plan_destroy(tnfa_eval_plan* plan);

/* ---- integration -------------------------------------------------------- */

/* Left Riemann sum over [0,1)^n: contract every site leg with the uniform
 * vector 1/base (1 when take_sum != 0) and contract the tree.  Replaces
 * integrate(f) (src/integration.jl:6-17).  out: 1 double (real) or 2 (complex),
 * host memory. */
int tnfa_integrate(tnfa_ctx* ctx, const tnfa_net* net, int take_sum, double* out);

/* <sum| O |f>: integral of O*f.  Replaces integrate(op, f) (src/integration.jl:20-32). */
int tnfa_integrate_operator(tnfa_ctx* ctx, const tnfa_net* op, const tnfa_net* net, int take_sum,
                            double* out);

/* Contract the site legs of variables vars[0..n_vars) with the uniform
 * vector (1/base, or 1 when take_sum) and, with merge_vertices, absorb every
 * vertex left without legs into its first neighbour (a vertex with no
 * neighbour left multiplies its scalar into the first vertex that still has
 * legs).  Replaces
 * partial_integrate (src/integration.jl:35-54) with merge_internal_tensors
 * (src/utils.jl:99-113).  "First" follows vertex_rank (one int per vertex,
 * e.g. the position in the caller's vertex order; NULL: the layout order).
 * The survivors are numbered breadth first, roots and neighbours in rank
 * order; out_vertex_of (sized n_vertices of net, may be NULL) receives the
 * input vertex of every output vertex.  Integrating every variable is an
 * error (use tnfa_integrate).  FP64 and complex128. */
int tnfa_partial_integrate(tnfa_ctx* ctx, const tnfa_net* net, int32_t n_vars, const int32_t* vars,
                           int take_sum, int merge_vertices, const int32_t* vertex_rank,
                           tnfa_net** out, int32_t* out_vertex_of);
/* Topology of a network (arrays sized by tnfa_net_info's n_vertices and the
 * leg count returned in *n_legs_total). Any pointer may be NULL. */
int tnfa_net_topology(const tnfa_net* net, int32_t* parent, int32_t* link_dim, int32_t* n_legs,
                      int32_t* leg_dim, int32_t* leg_var, int32_t* leg_digit, int32_t* leg_kind,
                      int32_t* n_legs_total);

/* ---- network algebra ---------------------------------------------------- */

/* Direct sum: f + g (bond dims add).  Replaces ITensorNetworks' add used by
 * `+` (src/elementary_functions.jl:67,82,99,119,134; semantics as
 * src/fixes.jl:39-91).  Same topology and legs required. */
int tnfa_add(tnfa_ctx* ctx, const tnfa_net* f, const tnfa_net* g, tnfa_net** out);
/* Pointwise product f * g (bond dims multiply).  Replaces multiply
 * (src/elementary_operators.jl:260-292). */
int tnfa_multiply(tnfa_ctx* ctx, const tnfa_net* f, const tnfa_net* g, tnfa_net** out);
/* diag(f) as an operator network (legs base^2).  Replaces operator_proj
 * (src/elementary_operators.jl:247-258). */
int tnfa_operator_proj(tnfa_ctx* ctx, const tnfa_net* f, tnfa_net** out);
/* Forest union: g's vertices appended after f's (the product of two
 * functions of disjoint vertex sets).  Replaces the disjoint-vertex branch of
 * multiply (src/elementary_operators.jl:263-270). */
int tnfa_net_concat(tnfa_ctx* ctx, const tnfa_net* f, const tnfa_net* g, tnfa_net** out);
/* Broadcast gather into another layout: output vertex t (of `target`) takes
 * its tensor from input vertex src_vertex[t], or is all ones when it is -1;
 * output axis a of t (its site legs one by one, then the parent bond, then
 * the child bonds) advances the input index by strides[a] elements (0
 * broadcasts: a leg or bond the input lacks).  Strides are listed vertex after
 * vertex.  Lifts a factor onto the union tree for multiply on partially
 * overlapping vertex sets (the shared-vertex branch of
 * src/elementary_operators.jl:260-281), and re-roots or renumbers a tree. */
int tnfa_net_gather(tnfa_ctx* ctx, const tnfa_net* f, const tnfa_topology* target,
                    const int32_t* src_vertex, const int64_t* strides, tnfa_net** out);
/* Element-type conversion: F64 <-> F32, F64 -> C128, F32 -> C128. */
int tnfa_net_convert(tnfa_ctx* ctx, const tnfa_net* f, int dtype, tnfa_net** out);

/* ---- operator construction ----------------------------------------------- */

/* Boundary conditions of the shift operators (src/elementary_operators.jl:32-57). */
typedef enum { TNFA_BC_DIRICHLET = 0, TNFA_BC_NEUMANN = 1, TNFA_BC_PERIODIC = 2 } tnfa_boundary;

/* A sum of product terms as an operator network on the tree of `topo` (a
 * function topology: digit legs of kind REAL or IMAG).  Term t has
 * coefficient coefs[t] and n_factors[t] site factors, listed term after term:
 * factor k acts on leg factor_leg[k] (index into topo's leg arrays) with the
 * leg_dim x leg_dim matrix M[out][in] that follows in factor_mat (row-major,
 * matrices back to back); legs without a factor carry the identity.  The
 * terms form a direct sum (bond = number of terms, coefficients on vertex 0)
 * compressed on the device by truncation with the relative cutoff, 64 terms
 * at a time.  Replaces ITensorNetworks' ttn(OpSum, s; cutoff) as the
 * reference calls it (src/elementary_operators.jl:114,119,151).  FP64. */
int tnfa_op_from_terms(tnfa_ctx* ctx, const tnfa_topology* topo, int32_t n_terms, const double* coefs,
                       const int32_t* n_factors, const int32_t* factor_leg, const double* factor_mat,
                       double cutoff, tnfa_net** op);
/* Finite-difference stencil along variable `dim` (base-2 digits) as an
 * operator network: weights[5] multiply f(x + 2d), f(x + d), f(x), f(x - d),
 * f(x - 2d); the forward shifts use right_bc and the backward ones left_bc
 * (tnfa_boundary); scale != 0 multiplies every vertex with a digit of `dim`
 * by 2^delta_power.  Replaces stencil (src/elementary_operators.jl:122-160)
 * and with weights (0, 1/2, 0, -1/2, 0), power 1 / (0, 1, -2, 1, 0), 2 /
 * (1/2, -1, 0, 1, -1/2), 3 / (1, -4, 6, -4, 1), 4 the first..fourth
 * derivative operators (:162-176); laplacian_operator (:178-189) is the
 * tnfa_add of the second derivatives of each variable. */
/* The stencil's product terms without building the operator (no context, no
 * device): the layout tnfa_op_from_terms takes (2 x 2 factor matrices), the
 * identity term first, before the 2^delta_power vertex scaling.  *n_terms
 * and *n_factors_total always receive the counts; the arrays are filled only
 * when max_terms / max_factors are large enough (call once with 0 to size
 * them). */
int tnfa_op_stencil_terms(const tnfa_topology* topo, int32_t dim, const double* weights, int32_t left_bc,
                          int32_t right_bc, int32_t max_terms, int32_t max_factors, double* coefs,
                          int32_t* n_factors, int32_t* factor_leg, double* factor_mat, int32_t* n_terms,
                          int32_t* n_factors_total);
int tnfa_op_build_stencil(tnfa_ctx* ctx, const tnfa_topology* topo, int32_t dim, const double* weights,
                          int32_t delta_power, int32_t left_bc, int32_t right_bc, int32_t scale,
                          double cutoff, tnfa_net** op);

/* ---- interpolation ------------------------------------------------------- */

/* Cross approximation (adaptive cross with full pivoting) of one sampled
 * block M (rows x cols, row-major FP64, host or device memory per `mem`):
 * repeatedly the entry of largest magnitude of the residual (the smallest
 * flat index among equal ones) becomes a pivot unless it is at most
 * tol * max|M|, and the residual loses its rank-one cross; at most maxrank
 * pivots.  piv_rows / piv_cols receive the pivots in order (room for
 * min(maxrank, rows, cols)), *rank their number, err[0] the largest residual
 * entry left (the rejected pivot, or the whole residual's maximum when the
 * rank cap was reached) and err[1] = max|M|.  The factorisation step of the
 * two-site tensor cross interpolation that ITensorTCI runs for the
 * reference's TCI extension (ext/ITensorNumericalAnalysisTCIExt/
 * tci_util.jl:21-55). */
int tnfa_cross(tnfa_ctx* ctx, const double* block, int mem, int32_t rows, int32_t cols, double tol,
               int32_t maxrank, int32_t* piv_rows, int32_t* piv_cols, int32_t* rank, double* err);

/* ---- operator application and truncation -------------------------------- */

/* y = O f, contracted exactly site by site then truncated with `params`.
 * Replaces operate (src/elementary_operators.jl:294-319), which calls
 * ITensorNetworks.contract(O, f; alg="fit", cutoff, maxdim, normalize). */
int tnfa_apply(tnfa_ctx* ctx, const tnfa_net* op, const tnfa_net* f,
               const tnfa_trunc_params* params, tnfa_net** out);
/* y = O f contracted exactly site by site, without truncation (every bond
 * of y is the operator's bond times f's).  The exact part of operate
 * (src/elementary_operators.jl:294-299) before ITensorNetworks' fit
 * compresses it; the forward map of tnfa_apply_vjp.  FP64 / complex128. */
int tnfa_apply_exact(tnfa_ctx* ctx, const tnfa_net* op, const tnfa_net* f, tnfa_net** out);
/* Vector-Jacobian product of tnfa_apply_exact with respect to f's tensors:
 * df += J^T dy, i.e. df_v[s_in][..] += sum O_v[(s_out, s_in)][..] dy_v[s_out][..]
 * with dy in the canonical layout of y = tnfa_apply_exact(op, f) and df in
 * f's (both n_elements scalars of f's type, host or device memory; complex
 * networks get the holomorphic derivative, not conjugated).  No reference
 * counterpart (the reference has no AD); it backs the rrule of operate,
 * differentiating through the exact contraction (not the truncation). */
int tnfa_apply_vjp(tnfa_ctx* ctx, const tnfa_net* op, const tnfa_net* f, const void* dy,
                   int dy_memory, void* df, int df_memory);
/* Batched form: n independent (op[i], f[i]) pairs of uneven shapes in one
 * scheduled pass. */
int tnfa_apply_batched(tnfa_ctx* ctx, int32_t n, const tnfa_net* const* ops,
                       const tnfa_net* const* fs, const tnfa_trunc_params* params,
                       tnfa_net** outs);
/* QR-orthogonalise toward the root(s), then SVD-truncate every bond with
 * `params`.  Replaces truncate (src/itensornetworkfunction.jl:114-118). */
int tnfa_truncate(tnfa_ctx* ctx, const tnfa_net* f, const tnfa_trunc_params* params,
                  tnfa_net** out);
/* Same for n networks at once. */
int tnfa_truncate_batched(tnfa_ctx* ctx, int32_t n, const tnfa_net* const* fs,
                          const tnfa_trunc_params* params, tnfa_net** outs);
/* Inner product <f|g> (conjugating f) and 2-norm.  out: 1 or 2 doubles. */
int tnfa_inner(tnfa_ctx* ctx, const tnfa_net* f, const tnfa_net* g, double* out);

/* ---- linear solve -------------------------------------------------------- */

typedef struct {
  int32_t nsweeps;      /* maximum number of sweeps                               */
  int32_t maxdim;       /* bond cap of the solution                               */
  double cutoff;        /* truncation of the two-site updates                     */
  double tol;           /* stop when ||A x - b|| / ||b|| <= tol                   */
  int32_t krylov_dim;   /* reserved (local systems: dense LU; GMRES(40) above it) */
  int32_t precision;    /* reserved (FP64)                                        */
  double a0, a1;        /* solve (a0 + a1*A) x = b                                */
  int32_t refinements;  /* iterative-refinement steps after the sweeps            */
  double refine_cutoff; /* truncation of residuals and corrections in refinement  */
} tnfa_linsolve_params;

/* Solve (a0 + a1 A) x = b on a tree with one site leg per vertex by
 * two-site updates (a path by alternating sweeps, any other tree by a
 * depth-first tour that updates every edge twice per sweep; each two-site
 * system by dense FP64 LU, or matrix-free GMRES(40) when large; truncated SVD
 * split); x0 seeds the sweep.  Then up to `refinements` steps of iterative refinement: r = b -
 * (a0 + a1 A) x formed exactly and truncated with refine_cutoff, the same
 * sweeps solve for a correction e, x <- truncate(x + e, refine_cutoff).
 * Replaces ITensorNetworks.linsolve as named for the Laplace solve
 * (examples/2d_laplace_solver.jl:33-34 uses the same sweep machinery through
 * dmrg).  rel_residual receives the final ||(a0 + a1 A) x - b|| / ||b||
 * computed exactly in FP64. */
int tnfa_linsolve(tnfa_ctx* ctx, const tnfa_net* A, const tnfa_net* b, const tnfa_net* x0,
                  const tnfa_linsolve_params* params, tnfa_net** x, double* rel_residual);

typedef struct {
  int32_t nsweeps;      /* maximum number of sweeps                               */
  int32_t maxdim;       /* bond cap of the state                                  */
  double cutoff;        /* truncation of the two-site updates                     */
  double tol;           /* stop when the energy changes by <= tol (relative)     */
  int32_t krylov_dim;   /* Lanczos vectors per restart (0: 30)                    */
  int32_t restarts;     /* Lanczos restarts per two-site update                   */
} tnfa_dmrg_params;

/* Lowest eigenpair of a symmetric operator H on a tree with one site leg per
 * vertex by two-site DMRG updates (a path by alternating sweeps, any other
 * tree by a depth-first tour): the two-site operator is applied densely on the
 * device or matrix-free for large systems, Lanczos (full
 * re-orthogonalisation, restarts) finds its lowest eigenvector,
 * a truncated SVD splits it, and the state is kept normalised.  Replaces
 * ITensorNetworks.dmrg as called by examples/2d_laplace_solver.jl:33-34
 * (nsites = 2, normalize = true).  energy receives the final eigenvalue. */
int tnfa_dmrg(tnfa_ctx* ctx, const tnfa_net* H, const tnfa_net* psi0, const tnfa_dmrg_params* params,
              tnfa_net** psi, double* energy);

/* ---- differentiation ----------------------------------------------------- */

/* Vector-Jacobian product of batched evaluation: dtensors += sum_p dout[p] *
 * d f(x_p) / d tensors (dout: n_points doubles; dtensors: n_elements scalars of
 * the network's type in canonical layout, accumulated into).  Computed in the
 * network's type (FP64, FP32 or complex128; for complex networks the result is
 * the holomorphic derivative sum_p dout_p d f_p / d T, not conjugated).  No
 * reference counterpart (the reference has no AD); it backs the rrule of
 * evaluate. */
int tnfa_evaluate_vjp(tnfa_ctx* ctx, const tnfa_net* net, const double* X, int64_t n_points,
                      int32_t n_dims, const int32_t* dims, int x_memory, const double* dout,
                      int dout_memory, void* dtensors, int dtensors_memory);

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif

#ifdef __cplusplus
}
#endif

#endif /* TNFA_H */
