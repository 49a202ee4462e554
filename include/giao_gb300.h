/*
 * giao_gb300.h -- C ABI of the GB300 electron-repulsion library.
 *
 * Plain pointers and sizes only.  Complex values are interleaved
 * (re, im) doubles, i.e. the memory layout of C99 double complex, NumPy
 * complex128 and std::complex<double>.  Every entry point returns 0 on
 * success or a negative gx_status; the message of the last failure on the
 * calling thread is returned by gx_last_error().
 *
 * Each entry point replaces one native function of the reference library
 * (simenkva/GIAOINT v0.11.1); the reference interface is cited beside it.
 * A Python binding over this ABI (ctypes) mirrors the reference's
 * pybind11 module names and argument meaning.
 */
#ifndef GIAO_GB300_H
#define GIAO_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  The Python layer maps them to the reference's exception
 * types (src/bindings.cpp:290-291 and pybind11's standard translation). */
enum gx_status {
    GX_OK = 0,
    GX_EINVAL = -1,   /* std::invalid_argument  -> ValueError              */
    GX_ERANGE = -2,   /* std::out_of_range      -> IndexError              */
    GX_ELENGTH = -3,  /* std::length_error      -> ValueError              */
    GX_EBOYS = -4,    /* giao::BoysNumericalError                          */
    GX_ECUDA = -5,    /* CUDA runtime failure   -> RuntimeError            */
    GX_ENOMEM = -6,   /* device memory budget   -> MemoryError             */
    GX_EPSD = -7,     /* Cholesky residual lost positive semidefiniteness  */
    GX_ETIMEOUT = -8, /* a bounded device wait gave up                     */
    GX_ECONSUMER = -9 /* a quartet consumer returned non-zero              */
};

/* Arithmetic of the quartet kernels. */
/* Arithmetic of the quartet kernels.  Both modes skip primitive quartets
 * whose Schwarz product B_P B_Q is negligible (below 1e-18 in FP64 mode,
 * 1e-15 in mixed mode); mixed mode evaluates those under `mixed_cutoff` in
 * FP32 (FP64 Boys function, FP32 recurrence and contraction, FP64 final
 * summation). */
enum gx_precision {
    GX_PRECISION_FP64 = 0,
    GX_PRECISION_MIXED = 1,
    GX_PRECISION_FP64_EXACT = 2  /* FP64, every primitive quartet (no screening) */
};

typedef struct gx_context gx_context; /* one device, its streams, Boys table, pools */
typedef struct gx_basis gx_basis;     /* shells resident on the device            */

typedef struct gx_eri_stats {
    int64_t requested;  /* quartets asked for                                  */
    int64_t computed;   /* quartets evaluated                                  */
    int64_t screened;   /* quartets dropped by Schwarz screening               */
    int64_t primitive_quartets; /* primitive quartets evaluated (all precisions) */
    int64_t fp32_primitive_quartets; /* of which in FP32 (mixed precision)       */
    int64_t skipped_primitive_quartets; /* dropped under the mixed-mode floor    */
    double kernel_ms;   /* device time of the quartet kernels                  */
    double prepare_ms;  /* host time from entry to the first launch (hashing,
                           screening, plan lookup or build)                     */
    double copy_ms;     /* device time of the output copy to host memory after
                           the quartet kernels (copies made while the classes
                           run are in kernel_ms)                                */
    double call_ms;     /* wall time of the call                               */
} gx_eri_stats;

/* ---------------------------------------------------------------------- */
/* context                                                                 */
/* ---------------------------------------------------------------------- */

/* Create a context on CUDA device `device`; builds the Boys tables. */
int gx_context_create(int device, gx_context** out);
void gx_context_destroy(gx_context* ctx);
/* Message of the last failure on the calling thread ("" if none). */
const char* gx_last_error(void);
/* Library version string. */
const char* gx_version(void);

/* ---------------------------------------------------------------------- */
/* host-side input model                                                   */
/* ---------------------------------------------------------------------- */

/* primitive_normalization (include/giao_integrals/types.hpp:141-142). */
double gx_primitive_normalization(double exponent, int lx, int ly, int lz);

/* Shell contraction normalisation as in the Shell constructor
 * (src/types.cpp:92-159): validates and writes coefs_out[ncontr][nprim].
 * normalize = 0 copies the coefficients unchanged after validation. */
int gx_shell_normalize(int l, int nprim, int ncontr, const double* exponents, const double* coefs_in,
                       int normalize, double* coefs_out);

/* Upload a basis (Basis, include/giao_integrals/types.hpp:108-124).
 * centers[3*ns]; exponents concatenated per shell; coefs concatenated,
 * contraction-major [ncontr][nprim] per shell, already normalised.
 * raw_primitives[s] != 0 omits the Cartesian primitive normalisation of
 * shell s (used by gx_primitive_eri for unnormalised primitives); may be NULL. */
int gx_basis_create(gx_context* ctx, int nshell, const double* centers, const int* l, const int* nprim,
                    const int* ncontr, const double* exponents, const double* coefs, const int* raw_primitives,
                    gx_basis** out);
void gx_basis_destroy(gx_basis* basis);
int64_t gx_basis_ao_count(const gx_basis* basis);

/* ---------------------------------------------------------------------- */
/* complex Boys function                                                   */
/* ---------------------------------------------------------------------- */

/* F_0..F_nmax(z) (or e^z F_n when scaled) for `count` arguments:
 * compute_boys (src/boys.cpp:245-294, bindings.cpp:444-482).
 * z[2*count]; out[2*count*(nmax+1)] row-major per argument; region[count]
 * receives the reference's region classification (BoysRegion order:
 * 0 power series, 1 adaptive quadrature, 2 scaled quadrature,
 * 3 positive asymptotic) and may be NULL.  Domain failures return GX_EBOYS
 * with the reference's message. */
int gx_boys(gx_context* ctx, const double* z, int64_t count, int nmax, int scaled, double* out, int* region);

/* ---------------------------------------------------------------------- */
/* electron-repulsion integrals                                            */
/* ---------------------------------------------------------------------- */

/* One primitive quartet with explicit Cartesian powers:
 * primitive_eri (src/eri.cpp:438-452, bindings.cpp:599-614).
 * exps[4], centers[12], angular[12], coefs[4], normalized[4], B[3], O[3]. */
int gx_primitive_eri(gx_context* ctx, const double* exps, const double* centers, const int* angular,
                     const double* coefs, const int* normalized, const double* B, const double* O, double* out);

/* Shell-quartet blocks packed in input order:
 * evaluate_eri_shell_quartets + append_eri_block
 * (src/eri.cpp:644-767, bindings.cpp:267-284, 672-731).
 * quartets[4*nq] shell indices; B[3], O[3] the field and gauge origin.
 * Screened quartets (Schwarz bound product < screening_threshold) are
 * omitted; kept[4*nkept] receives the emitted quartets, offsets[nkept+1]
 * the complex-element offsets of their blocks, out the values
 * (host memory, capacity out_capacity complex elements).
 * precision: gx_precision; mixed_cutoff the FP32 bound cutoff. */
int gx_eri_batch(gx_context* ctx, gx_basis* basis, const double* B, const double* O, const uint32_t* quartets,
                 int64_t nq, int precision, double mixed_cutoff, double screening_threshold, uint32_t* kept,
                 int64_t* offsets, double* out, int64_t out_capacity, gx_eri_stats* stats);

/* Same, with the packed values written to device memory `out_device`
 * (in-process GPU consumers; no host copy). */
int gx_eri_batch_device(gx_context* ctx, gx_basis* basis, const double* B, const double* O,
                        const uint32_t* quartets, int64_t nq, int precision, double mixed_cutoff,
                        double screening_threshold, uint32_t* kept, int64_t* offsets, void* out_device,
                        int64_t out_capacity, gx_eri_stats* stats);

/* One evaluated shell quartet, as the reference's ShellQuartetBlockView
 * (include/giao_integrals/eri.hpp:64-68): the shells as given, the AO counts
 * (na, nb, nc, nd) and `count` = na*nb*nc*nd interleaved complex128 values
 * in C order.  `values` points into a host buffer of the call and is valid
 * only while the consumer runs. */
typedef struct gx_quartet_block {
    uint32_t shells[4];
    int64_t shape[4];
    const double* values;
    int64_t count;
} gx_quartet_block;

/* Consumer of evaluated quartets (eri.hpp:70).  A non-zero return stops the
 * evaluation: the call then returns GX_ECONSUMER after the device work in
 * flight has finished. */
typedef int (*gx_quartet_consumer)(const gx_quartet_block* block, void* user_data);

/* Streams the blocks of nq shell quartets to `consumer`, replacing
 * evaluate_eri_shell_quartets / for_each_eri_shell_quartet
 * (include/giao_integrals/eri.hpp:127-135, src/eri.cpp:637-767): quartets
 * whose Schwarz product is below screening_threshold are dropped, every other
 * quartet is passed to the consumer once, in input order, on the calling
 * thread.  The quartets are evaluated in chunks of about 2^23 complex
 * elements into two page-locked host buffers kept by the context: the device
 * evaluates chunk k + 1 while the consumer reads chunk k, so host memory
 * stays bounded for any nq.  A null consumer is GX_EINVAL ("ERI quartet
 * consumer must not be null", as the reference).  stats (may be NULL)
 * receives the counts of the whole call. */
int gx_eri_for_each(gx_context* ctx, gx_basis* basis, const double* B, const double* O, const uint32_t* quartets,
                    int64_t nq, int precision, double mixed_cutoff, double screening_threshold,
                    gx_quartet_consumer consumer, void* user_data, gx_eri_stats* stats);

/* ERI centre derivatives of nq shell quartets, replacing
 * compute_eri_derivative_blocks behind _eri_derivative_batch
 * (src/bindings.cpp:2255-2303, src/derivatives.cpp:556-640, 954-959):
 * block i, at offsets[i] (complex elements; the call writes the nq + 1
 * offsets), is the C-order complex (4, 3, na, nb, nc, nd) array
 * d/dR_{slot,axis} (ab|cd) of quartet i, slots in quartet order, London-phase
 * centre response included at fixed B and gauge origin.  Shells through
 * l = 15; combined angular order + 1 through 32.  out: host memory of
 * out_capacity complex elements.  kernel_ms (may be NULL) receives the
 * derived-integral kernel time. */
int gx_eri_center_derivatives(gx_context* ctx, gx_basis* basis, const double* B, const double* O,
                              const uint32_t* quartets, int64_t nq, int64_t* offsets, double* out,
                              int64_t out_capacity, float* kernel_ms);

/* ERI magnetic derivatives d/dB_b (ab|cd) of nq shell quartets at fixed
 * gauge origin, replacing compute_eri_magnetic_derivatives
 * (src/derivatives.cpp:88-106, 268-280, 961-966; eri_magnetic_derivatives_shell,
 * src/bindings.cpp:1326-1342): block i at offsets[i] is the C-order complex
 * (3, na, nb, nc, nd) array, b the field axis.  Same limits and arguments as
 * gx_eri_center_derivatives. */
int gx_eri_magnetic_derivatives(gx_context* ctx, gx_basis* basis, const double* B, const double* O,
                                const uint32_t* quartets, int64_t nq, int64_t* offsets, double* out,
                                int64_t out_capacity, float* kernel_ms);

/* Mixed field/centre second derivatives d2/dR_{slot,r} dB_b (ab|cd) of nq
 * shell quartets at fixed gauge origin, replacing
 * compute_eri_mixed_derivatives (src/derivatives.cpp:160-181, 232-259,
 * 968-973; eri_mixed_derivatives_shell, src/bindings.cpp:2155-2165): block i
 * at offsets[i] is the C-order complex (4, 3, 3, na, nb, nc, nd) array, index
 * (slot 3 + r) 3 + b.  Shells through l = 14, combined order + 2 through 32.
 * Builds derived bases of two levels (16 shells per shell of the basis):
 * meant for small bases such as the four shells of one quartet. */
int gx_eri_mixed_derivatives(gx_context* ctx, gx_basis* basis, const double* B, const double* O,
                             const uint32_t* quartets, int64_t nq, int64_t* offsets, double* out, int64_t out_capacity);

/* Per-atom contraction of ERI centre derivatives with fixed densities,
 * replacing detail::contract_eri_derivatives behind _contract_eri_derivative_batch
 * (src/assembly.cpp:87-158, bindings.cpp:2418-2456): for every canonical
 * quartet (an error otherwise) and each of its distinct orbit images, the
 * derivative (conjugated for the two reversed images) times
 *   sum_pairs P[nu,mu] Q[sig,lam] (coulomb) + sum_pairs P[nu,lam] Q[sig,mu]
 *   (exchange) + gamma[mu,nu,lam,sig]
 * is added to out[shell_atoms[slot shell]][axis], in quartet and slot order.
 * coulomb / exchange: npc / npx pairs of complex (n, n) matrices (P then Q);
 * gamma: n^4 values, complex (gamma_complex != 0) or real, may be NULL;
 * out: complex (natom, 3), accumulated (not cleared).  The derivative blocks
 * stay on the device, computed in batches of at most batch_elements complex
 * values (a single larger quartet alone). */
int gx_eri_derivative_contraction(gx_context* ctx, gx_basis* basis, const double* B, const double* O,
                                  const uint32_t* quartets, int64_t nq, const int64_t* shell_atoms, int natom,
                                  int npc, const double* coulomb, int npx, const double* exchange,
                                  const double* gamma, int gamma_complex, int64_t batch_elements, double* out);

/* Derivative-density Schwarz factors, replacing EriDerivativeSchwarzBounds
 * (src/derivatives.cpp:1307-1372, bindings.cpp:2242-2253): values[ns*ns]
 * receives the factor of every ordered shell pair (a, b) at a*ns + b, and
 * ordinary[ns*ns] (may be NULL) the ordinary ERI Schwarz factors of
 * gx_schwarz.  A quartet's derivative bound is
 * max(values[ab] ordinary[cd], ordinary[ab] values[cd]), padded by
 * (1 + 128 eps) and one ulp (src/derivatives.cpp:1374-1383). */
int gx_eri_derivative_schwarz(gx_context* ctx, gx_basis* basis, const double* B, const double* O, double* values,
                              double* ordinary);

/* Same, with the blocks written to device memory `out_device`. */
int gx_eri_center_derivatives_device(gx_context* ctx, gx_basis* basis, const double* B, const double* O,
                                     const uint32_t* quartets, int64_t nq, int64_t* offsets, void* out_device,
                                     int64_t out_capacity, float* kernel_ms);

/* One shell quartet (compute_eri, src/eri.cpp:454-585; bindings.cpp:616-639).
 * out: complex (na, nb, nc, nd) C order, host memory. */
int gx_eri_shell(gx_context* ctx, gx_basis* basis, int a, int b, int c, int d, const double* B, const double* O,
                 double* out);

/* Full symmetric nao^4 tensor (compute_eri_tensor, src/eri.cpp:777-847,
 * bindings.cpp:640-671).  out: host complex[n^4]. */
int gx_eri_full(gx_context* ctx, gx_basis* basis, const double* B, const double* O, int precision,
                double mixed_cutoff, double screening_threshold, double* out);

/* Shell-pair Schwarz factors (EriSchwarzBounds, src/eri.cpp:587-619,
 * bindings.cpp:409-425).  out[ns*ns]. */
int gx_schwarz(gx_context* ctx, gx_basis* basis, const double* B, const double* O, double* out);

/* ---------------------------------------------------------------------- */
/* Cholesky-selected integrals and the pivoted Cholesky driver            */
/* ---------------------------------------------------------------------- */

/* Diagonal of W: detail::cholesky_diagonal (src/cholesky.cpp:285-314,
 * bindings.cpp:2306-2314).  pairs[2*npairs] shell pairs a <= b; out[n*n]. */
int gx_cholesky_diagonal(gx_context* ctx, gx_basis* basis, const int64_t* pairs, int64_t npairs, const double* B,
                         const double* O, double* out);

/* Pivot columns: detail::cholesky_columns (src/cholesky.cpp:203-323,
 * bindings.cpp:2315-2330).  pivots[2*npiv] AO pairs sharing one shell
 * pair.  out: float64[npiv][n][n] when B == 0 exactly, else
 * complex128[npiv][n][n]. */
int gx_cholesky_columns(gx_context* ctx, gx_basis* basis, const int64_t* pivots, int64_t npiv, const double* B,
                        const double* O, double* out);

typedef struct gx_cholesky_options {
    double threshold;           /* stop when max residual <= max(threshold, floor) */
    double screening_threshold; /* Schwarz skip of initial diagonal blocks          */
    int64_t max_rank;           /* output capacity (rows); MemoryError beyond       */
    int pivot_batch_size;       /* local block-pivot policy; 1 = strict global      */
} gx_cholesky_options;

/* Streamed pivoted Cholesky of W[(mu,nu),(lam,sig)] = (nu mu|lam sig):
 * python/giao_integrals/cholesky.py:60-297 with the integrals, pivot search,
 * factor update and residual kept on the device.
 * vectors: host complex128[max_rank][n][n]; pivots: int64[max_rank][2].
 * *rank and *max_residual receive the result. */
int gx_cholesky(gx_context* ctx, gx_basis* basis, const double* B, const double* O,
                const gx_cholesky_options* options, double* vectors, int64_t* pivots, int64_t* rank,
                double* max_residual);

/* Work and device time of one factorisation. */
typedef struct gx_cholesky_stats {
    int64_t rank;                        /* pivots taken (on failure: when it stopped)          */
    int64_t block_evaluations;           /* pivot shell-pair column evaluations                 */
    int64_t column_entries;              /* raw column entries extracted (candidates x n^2)     */
    int64_t column_primitive_quartets;   /* FP64 primitive quartets of the column evaluations   */
    int64_t diagonal_primitive_quartets; /* FP64 primitive quartets of the diagonal             */
    int64_t column_cache_capacity;       /* raw columns the cache may hold (fitted to memory)   */
    int64_t chained_steps;               /* pivot steps taken on the device without a host round
                                            trip (their columns were cached)                    */
    double column_model_flops;           /* FP64 FLOP model of the column primitive quartets    */
    double column_ms;                    /* event-timed column evaluations + extraction         */
    double update_ms;                    /* event-timed factor update, residual and argmax      */
    double update_bytes;                 /* algorithmic bytes of the updates: L read once per
                                            pivot (rank rows), raw column, new row, residual     */
    double update_flops;                 /* 2 (real) or 8 (complex) x rank x n^2, summed        */
    double column_pool_bytes;            /* device bytes of the column slots                    */
    double seconds;                      /* wall time of the factorisation                      */
} gx_cholesky_stats;

/* The same factorisation with the factors kept on the device (the factor
 * state a serving loop keeps resident): options->max_rank is the rank limit
 * (the reference's max_bytes // row_bytes; MemoryError beyond it) and the
 * factor rows grow on the device as the rank grows, so no output capacity
 * has to be guessed.  Destroy with gx_cholesky_factors_destroy. */
typedef struct gx_cholesky_factors gx_cholesky_factors;
int gx_cholesky_factor(gx_context* ctx, gx_basis* basis, const double* B, const double* O,
                       const gx_cholesky_options* options, gx_cholesky_factors** out);
/* rank, n (AOs), max residual diagonal and 1 when the factors are real
 * (zero field or a single centre: stored as float64 on the device). */
int gx_cholesky_factors_info(const gx_cholesky_factors* factors, int64_t* rank, int64_t* nao,
                             double* max_residual, int* real);
/* vectors: host complex128[rank][n][n] (may be NULL); pivots: int64[rank][2] (may be NULL). */
int gx_cholesky_factors_copy(const gx_cholesky_factors* factors, double* vectors, int64_t* pivots);
/* Device address of the factor rows ([rank][n*n], float64 when real else
 * complex128) for in-process GPU consumers; valid until destroyed. */
const void* gx_cholesky_factors_device(const gx_cholesky_factors* factors);
int gx_cholesky_factors_stats(const gx_cholesky_factors* factors, gx_cholesky_stats* out);
void gx_cholesky_factors_destroy(gx_cholesky_factors* factors);
/* Statistics of the last factorisation on the context (also after a failure). */
int gx_cholesky_last_stats(gx_context* ctx, gx_cholesky_stats* out);


/* GIAO nuclear-attraction matrix out[mu][nu] (complex128, n x n, AO order
 * of the basis) = sum_C -Z_C <mu|1/|r - C||nu> over nnuc point charges
 * (charges[nnuc] > 0, centers[3*nnuc]).  Replaces
 * compute_nuclear_attraction_matrix (src/nuclear.cpp:304-330; bindings.cpp:
 * 578-600).  Shells through l = 11. */
int gx_nuclear_attraction(gx_context* ctx, gx_basis* basis, const double* B, const double* O, int nnuc,
                          const double* charges, const double* centers, double* out);

/* ---------------------------------------------------------------------- */
/* streams, plans and device-resident execution                            */
/* ---------------------------------------------------------------------- */

/* Enqueue all later device work of `ctx` on `stream` (a cudaStream_t);
 * NULL restores the context's own stream.  No reference counterpart: the
 * reference runs synchronously on host threads (src/eri.cpp:708-763). */
int gx_context_set_stream(gx_context* ctx, void* stream);
/* Wait for the context's stream and report any device status word. */
int gx_context_synchronize(gx_context* ctx);

/* Several requests -- each its own basis, field (B[3 r], O[3 r]) and
 * quartet list -- packed into one class-sorted execution: quartets of
 * uneven classes and contraction depths from all requests share each class
 * launch (evaluate_eri_shell_quartets, src/eri.cpp:644-767, called once per
 * request in the reference).  Every basis must belong to ctx.  For request
 * r, offsets[r] (nq[r] + 1) receives the packed offsets of its blocks and
 * values[r] (host, capacity[r] complex elements) its blocks, in the layout
 * gx_eri_batch gives that request alone (no screening).  Work units never
 * mix requests, so on a context with stable launch configurations (below)
 * each request's values are bit for bit those of the request packed alone.
 * kernel_ms (may be NULL): device time of the class launches. */
int gx_eri_batch_packed(gx_context* ctx, int nreq, gx_basis* const* bases, const double* B, const double* O,
                        const uint32_t* const* quartets, const int64_t* nq, int precision, double mixed_cutoff,
                        int64_t* const* offsets, double* const* values, const int64_t* capacity,
                        double* kernel_ms);
/* 1: plans built on ctx from now on choose launch configurations that do
 * not depend on how many tasks a class holds (no splitting of ket
 * components over extra warps for small classes), so a request gives the
 * same bits alone and in any pack; 0 (default): configurations sized to the
 * plan.  No reference counterpart (the reference has no batching across
 * requests). */
int gx_context_set_stable_launch(gx_context* ctx, int stable);

/* How host-output gx_eri_batch calls copy the blocks to page-locked host
 * memory.  parts = 0, the default: the SMs copy each class's blocks right
 * after the class's kernels, through the buffer's mapped address, so the
 * copy overlaps the evaluation of the other classes.  parts = 1: one copy
 * after the whole evaluation.  parts >= 2: `parts` contiguous input ranges,
 * the copy of each range overlapping the evaluation of the later ones;
 * first_share in [0, 1) is the first range's share of the output elements
 * (0: equal ranges), the other ranges share the rest equally. */
int gx_context_set_copy_parts(gx_context* ctx, int parts, double first_share);

/* A plan fixes a quartet list (its class-sorted task list and packed
 * offsets, offsets[nq+1]) so that it can be evaluated for many fields
 * without host work: the persistent batched form of
 * evaluate_eri_shell_quartets (src/eri.cpp:644-767). */
typedef struct gx_eri_plan gx_eri_plan;
int gx_eri_plan_create(gx_context* ctx, gx_basis* basis, const uint32_t* quartets, int64_t nq, int64_t* offsets,
                       gx_eri_plan** out);
/* tasks (segmented quartets), primitive quartets, FP64 FLOP-model total and
 * kernel launches per execution. */
int gx_eri_plan_info(const gx_eri_plan* plan, int64_t* tasks, int64_t* primitive_quartets, double* model_flops,
                     int* launches);
/* Enqueue the evaluation for field (B, O) into device memory out_device
 * (complex128, offsets from gx_eri_plan_create).  Asynchronous: call
 * gx_context_synchronize (or synchronise the stream) before reading. */
int gx_eri_plan_execute(gx_eri_plan* plan, const double* B, const double* O, int precision, double mixed_cutoff,
                        void* out_device);
/* Primitive quartets evaluated by the last execution (FP64 and FP32) and
 * the matching FP64-structured FLOP model totals (waits for the stream). */
int gx_eri_plan_counts(gx_eri_plan* plan, int64_t* fp64_quartets, int64_t* fp32_quartets, double* fp64_flops,
                       double* fp32_flops);
void gx_eri_plan_destroy(gx_eri_plan* plan);

/* Number of (la, lb, lc, ld) classes (one kernel launch each). */
int gx_eri_plan_class_count(const gx_eri_plan* plan);
/* Executions served by replaying the plan's CUDA graph so far (a plan is
 * captured on its second execution with the same stream, output, precision
 * and cutoff, and replayed from then on). */
int gx_eri_plan_graph_replays(const gx_eri_plan* plan);

/* Per-class timing of one execution (synchronous). */
typedef struct gx_class_profile {
    int la, lb, lc, ld;
    int64_t tasks;                 /* segmented shell quartets */
    int64_t primitive_quartets;    /* before screening */
    int64_t fp64_quartets;         /* evaluated in FP64 */
    int64_t fp32_quartets;         /* evaluated in FP32 (mixed precision) */
    double model_flops_per_quartet;
    float ms;                      /* event-timed kernel duration */
    int per_group;                 /* launch configuration: primitive quartets per warp unit (0 = default) */
    int warps_per_block, batch;    /* generic kernel: warps per block, phase-1 batch */
    int64_t groups;                /* warp work units */
    int kt, ct;                    /* generic kernel: ket-transform rows and bra-transform components per lane */
    int min_blocks;                /* generic kernel: register-budget variant (resident blocks) */
    int stream;                    /* generic kernel: 1 = per-entry recurrences (stream mode) */
} gx_class_profile;
int gx_eri_plan_profile(gx_eri_plan* plan, const double* B, const double* O, int precision, double mixed_cutoff,
                        void* out_device, gx_class_profile* out);
/* Autotune the launch configuration of every class for one precision mode:
 * each class is timed (best of `repeats`) over its candidate work-unit sizes,
 * warps per block and phase-1 batch sizes, and the fastest is kept for later
 * executions in that mode.  Writes out_device.  default_ms / tuned_ms: summed
 * class times before and after. */
int gx_eri_plan_autotune(gx_eri_plan* plan, const double* B, const double* O, int precision, double mixed_cutoff,
                         void* out_device, int repeats, double* default_ms, double* tuned_ms);

/* Launch configuration of one class, as the autotuner chooses it (a zero
 * field: the kernel's fixed fallback for that knob; an untuned plan runs
 * the per-class configuration that gx_eri_plan_get_config reports, by
 * angular-momentum class): primitive quartets per warp unit, warps per block
 * cap (<= 4), phase-1 batch cap (<= 32), ket-transform rows per lane (1, 2,
 * 4), bra-transform components per lane (1-4), register-budget variant (2
 * or 4 resident blocks), 1 = no shared staging, 1 = stream mode (per-entry
 * recurrences into a two-column buffer), 1 = no FP32 lane kernel (mixed
 * precision, classes with 3 <= L <= 4: the generic kernel then also takes
 * the FP32 primitive quartets).  Fields other than per_group apply to the
 * generic kernel only. */
typedef struct gx_class_config {
    int per_group, warps_per_block, batch, kt, ct, min_blocks, nostage, stream, nolane;
} gx_class_config;
/* Read / replace the configuration of every class (gx_eri_plan_class_count
 * entries) for one precision mode; a set configuration is used by later
 * executions in that mode (replaying a saved tuning, or pinning one). */
int gx_eri_plan_get_config(gx_eri_plan* plan, int precision, gx_class_config* out);
int gx_eri_plan_set_config(gx_eri_plan* plan, int precision, const gx_class_config* confs);

/* Canonical shell quartets of an ns-shell basis: the lexicographic
 * minimum of each finite-field orbit {(ab|cd), (cd|ab), (ba|dc)*, (dc|ba)*}
 * (canonicalize_shell_quartet, src/eri.cpp:414-429), in the enumeration
 * order of compute_eri_tensor (src/eri.cpp:825-843).  out[4*count] may be
 * NULL to count only; returns the count. */
int64_t gx_canonical_quartets(int ns, uint32_t* out);

/* Measured FP64 FMA throughput of the device (TFLOP/s) from a dependent-
 * chain probe kernel: the roofline denominator of the FP64-bound kernels. */
int gx_measure_fp64_peak(gx_context* ctx, double* tflops);
/* The same probe in FP32: the denominator of the FP32 term of the
 * mixed-precision roofline. */
int gx_measure_fp32_peak(gx_context* ctx, double* tflops);

/* ---------------------------------------------------------------------- */
/* allocation-free Cholesky step                                           */
/* ---------------------------------------------------------------------- */

/* Largest n*n (ordered AO pairs) the allocation-free step accepts. */
#define GX_NOALLOC_MAX_ENTRIES 65536

typedef struct gx_cholesky_step_result {
    double max_residual; /* largest residual diagonal after the step (pivot zeroed) */
    int64_t argmax;      /* its flat index mu*n+nu, lowest index on ties            */
    double min_residual; /* smallest residual before clamping (PSD check)           */
} gx_cholesky_step_result;

/* One pivot step of the pivoted Cholesky that allocates no device memory
 * and needs no context: new_row = (column - conj(factors[:rank, pivot])
 * factors[:rank]) / sqrt(residual[pivot]) (symmetrised first when real),
 * residual -= |new_row|^2, clamped at 0 with the pivot zeroed, and the next
 * argmax and the PSD minimum written to `result`.  No counterpart in the
 * reference library: it is the device step of gx_cholesky offered to callers
 * that cannot let a library call cudaMalloc/cudaFree (they own all device
 * memory, e.g. through a pooling allocator or a hard memory cap, and cannot
 * afford the device-wide synchronisation those calls imply).
 * All pointers are device memory of the caller: factors [rank][n*n],
 * column [n*n], residual [n*n] float64, new_row [n*n], result one
 * gx_cholesky_step_result; values are float64 when real != 0, else
 * complex128.  Work is enqueued on `stream` (a cudaStream_t, NULL = default).
 * Scratch lives in a fixed device array of GX_NOALLOC_MAX_ENTRIES complex128
 * plus a few KiB, held by every GPU that loads the library until process
 * exit; n*n above GX_NOALLOC_MAX_ENTRIES returns GX_ELENGTH.  All calls share
 * that scratch, so calls that overlap on the GPU (different streams or
 * threads without ordering) race.  Every call outside stream capture looks
 * the scratch address up with the calling thread's current device (so a
 * context re-created after cudaDeviceReset is followed); a call under
 * capture reuses the address of the last uncaptured call on that device, so
 * the first call on a device must come before any stream capture.  The pivot
 * must have a positive residual (residual[pivot] > 0), as the allocating
 * driver guarantees; otherwise the row and result->min_residual are not
 * finite. */
int gx_cholesky_step_noalloc(const void* factors, int64_t rank, int64_t pivot, const void* column, int n, int real,
                             double* residual, void* new_row, void* result, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* GIAO_GB300_H */
