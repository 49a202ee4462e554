// Internal declarations shared by the host orchestration (gx_api.cu) and the
// kernels (gx_kernels.cu).  Not part of the C ABI.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "gx_device.cuh"

namespace gx {

// Device view of one angular-momentum pair class (la, lb): for every
// Cartesian component pair ab = ca * ncart(lb) + cb, the box of complex
// Hermite coefficients E~[k][l][m], k <= ax+bx, l <= ay+by, m <= az+bz,
// stored x-major at boxoff[ab] inside each primitive pair's record.
struct PairClassDev {
    int la, lb, nab, Lab, Etot;
    const int* boxoff;     // [nab]
    const int* boxdim;     // [nab] bx | by << 8 | bz << 16
    const uint32_t* ent;   // [Etot] k | l << 8 | m << 16
};

// One shell-quartet work item (segmented shells) and where its block goes.
struct Task {
    int sa, sb, sc, sd;
    long long out_off;  // complex-element offset of element (0,0,0,0)
    int st[4];          // complex-element strides of the component indices
    int pab, pcd;       // first primitive-pair record (sorted order) of the bra pair (sa, sb) and ket pair (sc, sd)
};

// Per-(basis, field) primitive-pair data, structure of arrays.
struct PairData {
    int npp;
    const double* p;       // [npp] exponent sum
    const double* Pr;      // [3*npp] product centre
    const double* Pi;      // [3*npp] imaginary part of the complex centre, -q/(2p)
    const double2* F;      // [npp] complex prefactor (coefficients, norms, K_ab, London phase, 1/p)
    const long long* Eoff; // [npp] offset of the primitive pair's E~ record in Epool
    const double2* Epool;  // complex Hermite coefficients
    const double* bound;   // [npp] primitive Schwarz factor sqrt(max |(ab|ba)_PP|)
    const float2* Epool32; // the same coefficients in FP32 (mixed precision)
    const int* order;      // [npp] records of each shell pair sorted by decreasing bound
    const float* sbound;   // [npp] bound of order[i] (FP32, for gating)
    const float4* g32;     // [2*npp] (P, p) and (Im P', 0) in FP32, for classifying Boys arguments
};

// True when the Boys argument T of primitive quartet (ip, iq) lies in the
// FP32 asymptotic sector of boys_eval32 with a margin, judged from the FP32
// pair geometry (a misjudged quartet is still exact: seeds32 rechecks T in
// FP64 and the caller falls back to the FP64 Boys function).
__device__ __forceinline__ bool boys_asymptotic32(const PairData& pp, int ip, int iq, int L) {
    const float4 a = pp.g32[2 * ip], b = pp.g32[2 * iq];
    const float4 ai = pp.g32[2 * ip + 1], bi = pp.g32[2 * iq + 1];
    const float dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
    const float ex = ai.x - bi.x, ey = ai.y - bi.y, ez = ai.z - bi.z;
    const float rho = __fdividef(a.w * b.w, a.w + b.w);
    const float x = rho * (fmaf(dx, dx, fmaf(dy, dy, dz * dz)) - fmaf(ex, ex, fmaf(ey, ey, ez * ez)));
    const float y = 2.0f * rho * fmaf(dx, ex, fmaf(dy, ey, dz * ez));
    return x >= 2.0f * L + 25.0f && fabsf(y) <= 0.45f * x && (x * x + y * y <= 150.0f * 150.0f || x >= 2.0f * L + 61.0f);
}

struct BasisDev {
    int ns;
    const double* center;  // [3*ns]
    const int* l;
    const int* nprim;
    const int* primoff;
    const double* exps;
    const double* coefs;   // per primitive, contraction-normalised (segmented shells)
    const int* raw;        // 1: no Cartesian primitive normalisation
    const int* sp_off;     // [ns*ns] first primitive pair of ordered shell pair (a, b)
};

struct QuartetClass {
    PairClassDev bra, ket;
    int L, Nab, NL;        // total order, herm_count(Lab), herm_count(L)
    int B1, CH;            // phase-1 batch (primitive quartets), ket-component chunk
    int nchunk;            // ket chunks per task group, run by separate warps
    int coop;              // batches of at most this many entries use the warp-cooperative recurrence
    int minb;              // register budget variant of the kernel: 2 or 4 resident blocks
    int stage_e;           // words (complex) of the per-warp E~ staging buffer (0: read E~ from global memory)
    int tab_words;         // 32-bit words of the block-shared class tables (0: read them from global memory)
    int KT, CT;            // Hermite rows per lane in the ket transform, ket components per lane in the bra transform
    int stream;            // 1: phase 1 keeps only the seeds of the batch; each entry's R is built by the warp
                           //    into a two-column buffer right before its ket transform (small shared footprint)
    int no32;              // 1: leave the FP32 entries of a mixed-precision pass to the FP32 lane kernel
    int ntask;
    const Task* tasks;
    int ngroup;
    const int2* groups;  // (first task, task count) per warp work unit
};

struct EriDev {
    BasisDev basis;
    PairData pairs;
    BoysTable boys;
    const GLRules* gl;
    const uint32_t* herm_xyz;  // packed (k, l, m) of herm index, L <= 32
    const int2* rec_plan;      // Hermite recurrence steps of every L <= REC_PLAN_MAX (see rec_plan_entry)
    const int* rec_plan_off;   // [REC_PLAN_MAX + 2] first step of each L
    double2* out;
    DevStatus* status;
    float skip_cut;   // primitive quartets with bound product below this are skipped
    float fp32_cut;   // ... below this (and above skip_cut) run in FP32; 0 = FP64 only.
                      // The FP32 quartets use FP32 Boys values in the asymptotic
                      // sector and FP64 ones elsewhere, then the FP32 recurrence.
    unsigned long long* counters;  // [0] FP64, [1] FP32 primitive quartets evaluated (may be null)
};

// In-place descending-level Hermite recurrence as a step list per total order
// L (the order of hermite_rec): for n = L-1 .. 0, every multi-index of total
// degree d = L-n .. 1 (x-major), then the seed of level n.  A step is
//   x = dst | s1 << 16,
//   y = s2 | axis << 14 | coef << 16 | seed << 22 | n << 23,
// meaning col[dst] = X[axis] col[s1] + coef col[s2] (coef = power - 1, 0: no
// second term), or col[0] = seed[n] when the seed bit is set.
constexpr int REC_PLAN_MAX = 16;

// ---- launch wrappers (gx_kernels.cu) -------------------------------------

cudaError_t launch_boys_table(double2* S, double2* E0, const GLRules* gl, int* fail_count, cudaStream_t s);
cudaError_t launch_boys_values(const double2* z, long long count, int nmax, int scaled, const BoysTable& tab,
                               const GLRules* gl, double2* out, int* region, DevStatus* st, cudaStream_t s);
cudaError_t launch_pair_precompute(const BasisDev& basis, const double* B, const double* O, int npp, const int* pp_a,
                                   const int* pp_b, const int* pp_pa, const int* pp_pb, const int* pp_class,
                                   const PairClassDev* classes, double* p, double* Pr, double* Pi, double2* F,
                                   const long long* Eoff, double2* Epool, float2* Epool32, double* bound, float4* g32,
                                   const EriDev* dev_for_bounds, cudaStream_t s);
size_t quartet_smem_bytes(const QuartetClass& qc, int warps_per_block, bool mixed);
cudaError_t launch_quartets(const EriDev& dev, const QuartetClass& qc, int warps_per_block, int grid,
                            cudaStream_t s);
cudaError_t launch_offset_copy(int* dst, const int* src, long long n, int off, cudaStream_t s);
cudaError_t launch_offset_copy(long long* dst, const long long* src, long long n, long long off, cudaStream_t s);
// bytes (a multiple of 16, both addresses 16-byte aligned) from device memory
// to page-locked host memory through its mapped device address, by at most
// `blocks` blocks of 512 threads
cudaError_t launch_host_copy(void* dst_mapped, const void* src, long long bytes, int blocks, cudaStream_t s);
// the entries of the `ntask` tasks of class (la, lb, lc, ld) from the packed
// device output `src` to page-locked host memory (mapped address, 16-byte
// aligned) at the same offsets
cudaError_t launch_class_copy(const Task* tasks, int ntask, int la, int lb, int lc, int ld, const double2* src,
                              void* dst_mapped, int sms, cudaStream_t s);
cudaError_t launch_scatter_full(const double2* packed, const long long* block_off, const int* block_info, int nblocks,
                                long long n, double2* full, cudaStream_t s);

// nuclear attraction (gx_nuclear.cu)
cudaError_t launch_nuclear(const BasisDev& bs, const PairData& pp, const BoysTable& boys, const GLRules* gl,
                           const uint32_t* herm_xyz, const PairClassDev* classes, const int* pp_class, int nnuc,
                           const double* charge, const double* center, const long long* seg_ao, long long n,
                           int max_pair_L, int max_nab, double2* out, DevStatus* status, cudaStream_t s);

// ERI centre and magnetic derivatives (gx_deriv.cu): gathers the
// derived-basis blocks of nq quartets into (4, 3, na, nb, nc, nd) or
// (3, na, nb, nc, nd) blocks at out + offsets[i].
struct DerivCombineArgs {
    int nq;
    int mode;                        // 0: centre derivatives (12 per element), 1: magnetic (3 per element)
    int field;                       // centre mode with B != 0: U blocks and the plain block follow
    const uint32_t* quartets;        // [4 nq] original shells
    const long long* offsets;        // [nq + 1] output offsets (12 x block size each)
    const long long* derived_offsets;  // [nq] first derived block of each quartet
    const int* shell_l;              // per original shell
    const int* shell_ncontr;
    const int* shell_raw;
    const double* shell_center;      // [3 ns]
    const double* shell_inv2a;       // 1 / (2 alpha) of single-primitive shells, else 0: their U block
                                     // (centre mode) is omitted and read as Z / (2 alpha)
    const double2* derived;          // derived-basis ERI blocks
    double2* out;
    double B[3], O[3];
    double inv_sqrt_df[18];          // 1 / sqrt((2n - 1)!!)
};
cudaError_t launch_deriv_combine(const DerivCombineArgs& args, long long total, int sms, cudaStream_t s);
// Mixed field/centre derivatives (4, 3, 3, ...) assembled from the centre
// derivatives (D[0]: the quartets, D[1 + j]: the quartets with slot j
// replaced by its U shell) and the plain blocks (E at eoff[0 .. 4]).
struct DerivMixedArgs {
    int nq;
    const uint32_t* quartets;        // [4 nq] original shells
    const long long* offsets;        // [nq + 1] output offsets (36 x block size each)
    const long long* doff;           // [5 nq] centre-derivative block offsets per list
    const long long* eoff;           // [5 nq] plain block offsets per list
    const double2* D[5];
    const double2* E;
    const int* shell_l;
    const int* shell_ncontr;
    const int* shell_raw;
    const double* shell_center;
    double2* out;
    double O[3];
    double inv_sqrt_df[18];
};
cudaError_t launch_deriv_mixed(const DerivMixedArgs& args, long long total, int sms, cudaStream_t s);
// Twelve partial sums per canonical quartet of the per-atom contraction of
// centre derivatives with density pairs and a two-particle density.
struct DerivContractArgs {
    int nq;
    const uint32_t* quartets;        // [4 nq]
    const long long* offsets;        // [nq] derivative block offsets in D
    const double2* D;
    const int* shell_l;
    const int* shell_ncontr;
    const long long* ao_start;       // per shell
    long long n;                     // AO count
    int npc, npx;                    // Coulomb / exchange pairs
    const double2* coulomb;          // [2 npc] (n, n): P, Q, P, Q, ...
    const double2* exchange;         // [2 npx] (n, n)
    const double2* gamma;            // complex n^4 or null
    const double* gamma_real;        // real n^4 or null
    double2* partials;               // [nq][12]
};
cudaError_t launch_deriv_contract(const DerivContractArgs& args, int sms, cudaStream_t s);
// dst[i] = |src[idx[i]]| (diagonal elements of the derivative-bound blocks)
cudaError_t launch_gather_abs(const double2* src, const long long* idx, double* dst, long long n, int sms,
                              cudaStream_t s);

// FP32 lane kernel of the mixed-precision entries of 3 <= L <= 4 classes
// (gx_lane*.cu, dispatched in gx_small.cu); runs after the class-generic
// kernel of the same class on the same stream
bool lane32_class(int la, int lb, int lc, int ld);
cudaError_t launch_lane32(int la, int lb, int lc, int ld, const EriDev& d, const QuartetClass& qc, cudaStream_t s);

// register-resident small classes (gx_small.cu)
bool small_class(int la, int lb, int lc, int ld);
cudaError_t launch_small(int la, int lb, int lc, int ld, const EriDev& d, const QuartetClass& qc, cudaStream_t s);

// Cholesky (gx_chol.cu)
cudaError_t launch_chol_diag(const double2* packed, const long long* boff, const int* info, int nblocks, int n,
                             double* D, cudaStream_t s);
// flip (may be null): per block, 1 when it was evaluated as (sb sa | a b)
cudaError_t launch_chol_cols(bool real, const double2* packed, const long long* boff, const int* info,
                             const int* flip, int nblocks, const int* cand, int ncand, int nc, int nd, int n,
                             void* const* dst, cudaStream_t s);
cudaError_t launch_chol_scan(const double* res, long long N, void* partial, void* out, cudaStream_t s);
// gemv_partials (max_chunks x n^2 values, may be null): splits the factor
// update over rank chunks when that gives more blocks; sms: SM count.
cudaError_t launch_chol_step(bool real, const void* L, long long ld, int rank, long long piv, const void* column,
                             void* work, int n, double* res, double* scale, void* Lrow, void* partial, void* out,
                             cudaStream_t s, void* gemv_partials = nullptr, int max_chunks = 0, int sms = 0);
cudaError_t launch_chol_final_residual(bool real, const double* D, const void* L, int rank, long long N, double* res,
                                       cudaStream_t s);
// State of a chain of pivot steps taken on the device (launch_chol_chain).
struct ChainState {
    long long pivot;  // pivot of the current step
    int slot;         // its column slot in the cache
    int rank;         // factor rows so far
    int active;       // 1 while the chain runs
    int steps;        // steps taken by this chain
    int stop;         // why it stopped: 1 column not cached, 2 converged, 3 rank limit, 4 PSD check
    int rank_limit;   // rows the factor buffer (and the caller's limit) allows
    double scale;     // 1 / sqrt(residual) of the current pivot
    unsigned int done;  // blocks of the current update that have finished (0 between steps)
};
// Enqueue `steps` chained pivot steps (each returns at once after the chain
// stopped): pool holds the cached raw columns (slot_of[flat index] = slot,
// -1 if absent), log receives the pivot of every step at its rank.  Two
// launches per step: the rank-chunked GEMV, and the row/residual update,
// which sums the chunks, applies the scale chosen at selection, and whose
// last block reduces the residual and selects the next pivot.
cudaError_t launch_chol_chain(bool real, void* L, long long N, int n, int rank_hi, int steps, ChainState* st,
                              int* slot_of, long long* log, const void* pool, double* res, void* partial, void* out,
                              void* gemv_partials, int max_chunks, int sms, double tol, double psd, cudaStream_t s);
size_t chol_red_bytes();
// dst[i] = (src[i], 0) for i < n
cudaError_t launch_widen_real(const double* src, double2* dst, long long n, int sms, cudaStream_t s);
size_t chol_partial_bytes();

// record a failure for gx_last_error() and return its code (gx_api.cu)
int set_error(int code, const std::string& msg);

cudaError_t run_fp64_probe(int sms, cudaStream_t s, float* ms, double* flops);
cudaError_t run_fp32_probe(int sms, cudaStream_t s, float* ms, double* flops);

}  // namespace gx
