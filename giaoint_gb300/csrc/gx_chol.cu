// Device kernels of the streamed pivoted Cholesky (K6-K9):
//
//   chol_diag_kernel     (mu nu|nu mu) diagonal from packed (ab|ba) blocks,
//                        placed as src/cholesky.cpp:305-311
//   chol_cols_kernel     pivot columns (mu nu|p1 p0) from packed
//                        (ab|sb sa) blocks; zero-phase real path mirrored and
//                        same-shell averaged as src/cholesky.cpp:245-279
//   chol_gemv_kernel     column -= conj(L[:rank, piv]) L[:rank]
//                        (python/giao_integrals/cholesky.py:268)
//   chol_update_kernel   real symmetrisation, 1/sqrt(residual) scale, new
//                        factor row, residual -= |column|^2, PSD minimum,
//                        clamp, zeroed pivot and the next argmax, fused
//                        (cholesky.py:269-281)
//   argmax reductions    lowest flat index on ties (NumPy argmax order)
#include <algorithm>

#include "gx_internal.h"

namespace gx {

// ---- diagonal --------------------------------------------------------------

// info per block: ao_a, ao_b, na, nb
__global__ void chol_diag_kernel(const double2* packed, const long long* boff, const int* info, int nblocks, int n,
                                 double* D) {
    const int bi = blockIdx.x;
    if (bi >= nblocks) return;
    const int oa = info[4 * bi], ob = info[4 * bi + 1], na = info[4 * bi + 2], nb = info[4 * bi + 3];
    const double2* blk = packed + boff[bi];
    for (int e = threadIdx.x; e < na * nb; e += blockDim.x) {
        const int i = e / nb, j = e - i * nb;
        const double v = blk[(((long long)i * nb + j) * nb + j) * na + i].x;
        const long long mu = oa + i, nu = ob + j;
        D[nu * n + mu] = v;
        if (oa != ob) D[mu * n + nu] = v;
    }
}

cudaError_t launch_chol_diag(const double2* packed, const long long* boff, const int* info, int nblocks, int n,
                             double* D, cudaStream_t s) {
    if (nblocks <= 0) return cudaSuccess;
    chol_diag_kernel<<<nblocks, 128, 0, s>>>(packed, boff, info, nblocks, n, D);
    return cudaGetLastError();
}

// ---- columns ---------------------------------------------------------------

// info per block: ao_a, ao_b, na, nb, same_shell; cand[2*k] = (c, d) local
// indices in shells (sb, sa); dst[k] = column k (n*n values).  flip[block]
// (may be null): the block was evaluated as (sb sa | a b), laid out
// (nc, nd, na, nb), which equals (a b | sb sa) by the exchange of the two
// electrons.
template <bool REAL>
__global__ void chol_cols_kernel(const double2* packed, const long long* boff, const int* info, const int* flip,
                                 int nblocks, const int* cand, int ncand, int nc, int nd, int n, void* const* dst) {
    const int bi = blockIdx.x;
    if (bi >= nblocks) return;
    const int oa = info[5 * bi], ob = info[5 * bi + 1], na = info[5 * bi + 2], nb = info[5 * bi + 3];
    const bool same = info[5 * bi + 4] != 0;
    const bool flipped = flip != nullptr && flip[bi] != 0;
    const double2* blk = packed + boff[bi];
    const int per = na * nb;
    auto at = [&](int i, int j, int c, int d) -> double2 {
        return flipped ? blk[(((long long)c * nd + d) * na + i) * nb + j]
                       : blk[(((long long)i * nb + j) * nc + c) * nd + d];
    };
    for (int e = threadIdx.x; e < per * ncand; e += blockDim.x) {
        const int k = e / per, r = e - k * per;
        const int i = r / nb, j = r - i * nb;
        const int c = cand[2 * k], d = cand[2 * k + 1];
        const double2 v = at(i, j, c, d);
        const long long mu = oa + i, nu = ob + j;
        if (REAL) {
            double s = v.x;
            if (same) s = (s + at(j, i, c, d).x) * 0.5;
            double* out = static_cast<double*>(dst[k]);
            out[mu * n + nu] = s;
            if (!same) out[nu * n + mu] = s;
        } else {
            double2* out = static_cast<double2*>(dst[k]);
            out[mu * n + nu] = v;
        }
    }
}

cudaError_t launch_chol_cols(bool real, const double2* packed, const long long* boff, const int* info,
                             const int* flip, int nblocks, const int* cand, int ncand, int nc, int nd, int n,
                             void* const* dst, cudaStream_t s) {
    if (nblocks <= 0) return cudaSuccess;
    if (real)
        chol_cols_kernel<true><<<nblocks, 256, 0, s>>>(packed, boff, info, flip, nblocks, cand, ncand, nc, nd, n,
                                                       dst);
    else
        chol_cols_kernel<false><<<nblocks, 256, 0, s>>>(packed, boff, info, flip, nblocks, cand, ncand, nc, nd, n,
                                                        dst);
    return cudaGetLastError();
}

// ---- argmax / min reductions -------------------------------------------------

struct Red {
    double maxv;
    long long idx;
    double minv;
};

__device__ __forceinline__ void red_merge(Red& a, const Red& b) {
    if (b.maxv > a.maxv || (b.maxv == a.maxv && b.idx < a.idx)) {
        a.maxv = b.maxv;
        a.idx = b.idx;
    }
    a.minv = fmin(a.minv, b.minv);
}

__device__ Red block_reduce(Red r) {
    __shared__ Red sh[32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) {
        Red t;
        t.maxv = __shfl_down_sync(0xffffffffu, r.maxv, o);
        t.idx = __shfl_down_sync(0xffffffffu, r.idx, o);
        t.minv = __shfl_down_sync(0xffffffffu, r.minv, o);
        red_merge(r, t);
    }
    if (lane == 0) sh[w] = r;
    __syncthreads();
    if (w == 0) {
        r = lane < (int)(blockDim.x >> 5) ? sh[lane] : Red{-1.0 / 0.0, (long long)1 << 62, 1.0 / 0.0};
        for (int o = 16; o > 0; o >>= 1) {
            Red t;
            t.maxv = __shfl_down_sync(0xffffffffu, r.maxv, o);
            t.idx = __shfl_down_sync(0xffffffffu, r.idx, o);
            t.minv = __shfl_down_sync(0xffffffffu, r.minv, o);
            red_merge(r, t);
        }
    }
    return r;
}

constexpr int RED_BLOCKS = 256;

__global__ void chol_scan_kernel(const double* res, long long N, Red* partial) {
    Red r{-1.0 / 0.0, (long long)1 << 62, 1.0 / 0.0};
    for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < N; j += (long long)gridDim.x * blockDim.x) {
        const double v = res[j];
        red_merge(r, Red{v, j, v});
    }
    r = block_reduce(r);
    if (threadIdx.x == 0) partial[blockIdx.x] = r;
}

__global__ void chol_final_kernel(const Red* partial, int np, Red* out) {
    Red r{-1.0 / 0.0, (long long)1 << 62, 1.0 / 0.0};
    for (int i = threadIdx.x; i < np; i += blockDim.x) red_merge(r, partial[i]);
    r = block_reduce(r);
    if (threadIdx.x == 0) *out = r;
}

cudaError_t launch_chol_scan(const double* res, long long N, void* partial, void* out, cudaStream_t s) {
    chol_scan_kernel<<<RED_BLOCKS, 256, 0, s>>>(res, N, static_cast<Red*>(partial));
    chol_final_kernel<<<1, 256, 0, s>>>(static_cast<const Red*>(partial), RED_BLOCKS, static_cast<Red*>(out));
    return cudaGetLastError();
}

// ---- factor update -----------------------------------------------------------

// acc +/- conj(a) * b as four dependent-pair FMAs (the complex update is
// FP64-pipe bound: 4 DFMA per 16-byte element instead of 4 + 2 adds)
__device__ __forceinline__ double2 conj_mul_add(double2 acc, double2 a, double2 b) {
    return c2(fma(a.y, b.y, fma(a.x, b.x, acc.x)), fma(-a.y, b.x, fma(a.x, b.y, acc.y)));
}
__device__ __forceinline__ double2 conj_mul_sub(double2 acc, double2 a, double2 b) {
    return c2(fma(-a.y, b.y, fma(-a.x, b.x, acc.x)), fma(a.y, b.x, fma(-a.x, b.y, acc.y)));
}

template <typename T>
__global__ void chol_gemv_kernel(const T* L, long long ld, int rank, long long piv, const T* col_in, T* col_out,
                                 long long N) {
    __shared__ T coef[256];
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    T acc;
    if constexpr (sizeof(T) == 8) {
        acc = j < N ? col_in[j] : T(0);
    } else {
        acc = j < N ? col_in[j] : c2(0.0, 0.0);
    }
    for (int r0 = 0; r0 < rank; r0 += 256) {
        const int nr = min(256, rank - r0);
        __syncthreads();
        for (int i = threadIdx.x; i < nr; i += blockDim.x) coef[i] = L[(long long)(r0 + i) * ld + piv];
        __syncthreads();
        if (j < N) {
            // eight independent row loads in flight per thread: the GEMV is
            // bound by HBM bandwidth, not by load latency
#pragma unroll 8
            for (int r = 0; r < nr; ++r) {
                const T lv = __ldg(&L[(long long)(r0 + r) * ld + j]);
                if constexpr (sizeof(T) == 8) {
                    acc -= coef[r] * lv;
                } else {
                    acc = conj_mul_sub(acc, coef[r], lv);
                }
            }
        }
    }
    if (j < N) col_out[j] = acc;
}

// The same update with the rank split over blockIdx.y: block (x, y) sums
// conj(L[r, piv]) L[r, j] over its rows into partials[y][j], and
// chol_gemv_sum_kernel subtracts the chunks in order.  Small n (few column
// entries) otherwise leaves too few loads in flight to stream L at HBM speed.
template <typename T>
__global__ void chol_gemv_split_kernel(const T* L, long long ld, int rank, long long piv, int chunk, T* partials,
                                       long long N) {
    __shared__ T coef[256];
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int rbeg = blockIdx.y * chunk, rend = min(rank, rbeg + chunk);
    T acc;
    if constexpr (sizeof(T) == 8) {
        acc = T(0);
    } else {
        acc = c2(0.0, 0.0);
    }
    for (int r0 = rbeg; r0 < rend; r0 += 256) {
        const int nr = min(256, rend - r0);
        __syncthreads();
        for (int i = threadIdx.x; i < nr; i += blockDim.x) coef[i] = L[(long long)(r0 + i) * ld + piv];
        __syncthreads();
        if (j < N) {
#pragma unroll 8
            for (int r = 0; r < nr; ++r) {
                const T lv = __ldg(&L[(long long)(r0 + r) * ld + j]);
                if constexpr (sizeof(T) == 8) {
                    acc += coef[r] * lv;
                } else {
                    acc = conj_mul_add(acc, coef[r], lv);
                }
            }
        }
    }
    if (j < N) partials[(long long)blockIdx.y * N + j] = acc;
}

template <typename T>
__global__ void chol_gemv_sum_kernel(const T* col_in, const T* partials, int nchunks, long long N, T* col_out) {
    for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < N; j += (long long)gridDim.x * blockDim.x) {
        T acc = col_in[j];
        for (int y = 0; y < nchunks; ++y) {
            if constexpr (sizeof(T) == 8) {
                acc -= partials[(long long)y * N + j];
            } else {
                acc = csub(acc, partials[(long long)y * N + j]);
            }
        }
        col_out[j] = acc;
    }
}

// scale = 1/sqrt(residual[piv]) (read before the update)
__global__ void chol_scale_kernel(const double* res, long long piv, double* scale) { *scale = rsqrt(res[piv]); }

template <typename T>
__global__ void chol_update_kernel(const T* col, int n, long long piv, const double* scale, T* Lrow, double* res,
                                   Red* partial) {
    const long long N = (long long)n * n;
    const double sc = *scale;
    Red r{-1.0 / 0.0, (long long)1 << 62, 1.0 / 0.0};
    for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < N; j += (long long)gridDim.x * blockDim.x) {
        double mag2;
        if constexpr (sizeof(T) == 8) {
            const long long mu = j / n, nu = j - mu * n;
            const double c = (col[j] + col[nu * n + mu]) * 0.5 * sc;
            Lrow[j] = c;
            mag2 = c * c;
        } else {
            const double2 c = cscale(col[j], sc);
            Lrow[j] = c;
            mag2 = c.x * c.x + c.y * c.y;
        }
        const double nr = res[j] - mag2;
        const double kept = j == piv ? 0.0 : fmax(nr, 0.0);
        res[j] = kept;
        red_merge(r, Red{kept, j, nr});
    }
    r = block_reduce(r);
    if (threadIdx.x == 0) partial[blockIdx.x] = r;
}

cudaError_t launch_chol_step(bool real, const void* L, long long ld, int rank, long long piv, const void* column,
                             void* work, int n, double* res, double* scale, void* Lrow, void* partial, void* out,
                             cudaStream_t s, void* gemv_partials, int max_chunks, int sms) {
    const long long N = (long long)n * n;
    const int blocks = (int)((N + 127) / 128);
    // rank chunks: enough blocks for about eight per SM, at least 32 rows each
    int nchunks = 1;
    if (gemv_partials && max_chunks > 1 && rank >= 64 && sms > 0) {
        nchunks = std::max(1, std::min({max_chunks, (8 * sms) / std::max(blocks, 1), (rank + 31) / 32}));
    }
    if (nchunks > 1) {
        const int chunk = (rank + nchunks - 1) / nchunks;
        const dim3 grid(blocks, nchunks);
        const int sblocks = (int)std::min<long long>((N + 255) / 256, 8LL * sms);
        if (real) {
            chol_gemv_split_kernel<double><<<grid, 128, 0, s>>>(static_cast<const double*>(L), ld, rank, piv, chunk,
                                                                static_cast<double*>(gemv_partials), N);
            chol_gemv_sum_kernel<double><<<sblocks, 256, 0, s>>>(static_cast<const double*>(column),
                                                                  static_cast<const double*>(gemv_partials), nchunks,
                                                                  N, static_cast<double*>(work));
        } else {
            chol_gemv_split_kernel<double2><<<grid, 128, 0, s>>>(static_cast<const double2*>(L), ld, rank, piv, chunk,
                                                                 static_cast<double2*>(gemv_partials), N);
            chol_gemv_sum_kernel<double2><<<sblocks, 256, 0, s>>>(static_cast<const double2*>(column),
                                                                   static_cast<const double2*>(gemv_partials), nchunks,
                                                                   N, static_cast<double2*>(work));
        }
    } else if (real) {
        chol_gemv_kernel<double><<<blocks, 128, 0, s>>>(static_cast<const double*>(L), ld, rank, piv,
                                                        static_cast<const double*>(column),
                                                        static_cast<double*>(work), N);
    } else {
        chol_gemv_kernel<double2><<<blocks, 128, 0, s>>>(static_cast<const double2*>(L), ld, rank, piv,
                                                         static_cast<const double2*>(column),
                                                         static_cast<double2*>(work), N);
    }
    chol_scale_kernel<<<1, 1, 0, s>>>(res, piv, scale);
    if (real)
        chol_update_kernel<double><<<RED_BLOCKS, 256, 0, s>>>(static_cast<const double*>(work), n, piv, scale,
                                                              static_cast<double*>(Lrow), res,
                                                              static_cast<Red*>(partial));
    else
        chol_update_kernel<double2><<<RED_BLOCKS, 256, 0, s>>>(static_cast<const double2*>(work), n, piv, scale,
                                                               static_cast<double2*>(Lrow), res,
                                                               static_cast<Red*>(partial));
    chol_final_kernel<<<1, 256, 0, s>>>(static_cast<const Red*>(partial), RED_BLOCKS, static_cast<Red*>(out));
    return cudaGetLastError();
}

// ---- chained steps: pivots taken on the device while their columns are cached ----
//
// After a step the next pivot is the argmax of the residual.  When its raw
// column is already in the column cache (slot_of[pivot] >= 0), the next step
// needs no host decision, so the host enqueues up to K steps at once and
// synchronises once: chain_select_kernel takes the argmax of the previous
// step, stops the chain (active = 0, with the reason) when the residual has
// converged, the rank limit is reached, the PSD check failed or the column is
// not cached, and otherwise records the pivot and its slot; the step kernels
// below read the pivot, rank and column from that state and return at once
// when the chain has stopped.

// Select logic shared by the chain's first step and the fused end of every
// step: stop the chain, or take the argmax as the next pivot (its column
// slot, its scale 1/sqrt(residual), its place in the log).
__device__ void chain_select(ChainState* st, const Red& r, int* slot_of, long long* log, double tol, double psd) {
    int stop = 0;
    int slot = -1;
    if (r.minv < -psd)
        stop = 4;
    else if (!(r.maxv > tol))
        stop = 2;
    else if (st->rank >= st->rank_limit)
        stop = 3;
    else if ((slot = slot_of[r.idx]) < 0)
        stop = 1;
    if (stop) {
        st->active = 0;
        st->stop = stop;
        return;
    }
    st->pivot = r.idx;
    st->slot = slot;
    st->scale = rsqrt(r.maxv);  // r.maxv is the stored residual of the pivot
    slot_of[r.idx] = -1;
    log[st->rank] = r.idx;
}

__global__ void chain_select_kernel(ChainState* st, const Red* red, int* slot_of, long long* log, double tol,
                                    double psd) {
    if (!st->active) return;
    chain_select(st, *red, slot_of, log, tol, psd);
}

template <typename T>
__global__ void chain_gemv_split_kernel(const T* L, long long ld, const ChainState* st, int nchunks, T* partials,
                                        long long N) {
    if (!st->active) return;
    __shared__ T coef[256];
    const int rank = st->rank;
    const long long piv = st->pivot;
    const int chunk = (rank + nchunks - 1) / nchunks;
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int rbeg = blockIdx.y * chunk, rend = min(rank, rbeg + chunk);
    T acc;
    if constexpr (sizeof(T) == 8) {
        acc = T(0);
    } else {
        acc = c2(0.0, 0.0);
    }
    for (int r0 = rbeg; r0 < rend; r0 += 256) {
        const int nr = min(256, rend - r0);
        __syncthreads();
        for (int i = threadIdx.x; i < nr; i += blockDim.x) coef[i] = L[(long long)(r0 + i) * ld + piv];
        __syncthreads();
        if (j < N) {
#pragma unroll 8
            for (int r = 0; r < nr; ++r) {
                const T lv = __ldg(&L[(long long)(r0 + r) * ld + j]);
                if constexpr (sizeof(T) == 8) {
                    acc += coef[r] * lv;
                } else {
                    acc = conj_mul_add(acc, coef[r], lv);
                }
            }
        }
    }
    if (j < N) partials[(long long)blockIdx.y * N + j] = acc;
}

// Updated column entry j: the cached raw column minus the rank-chunk partial
// sums, in chunk order.
template <typename T>
__device__ __forceinline__ T chain_column(const T* col_in, const T* partials, int nchunks, long long N, long long j) {
    T acc = col_in[j];
    for (int y = 0; y < nchunks; ++y) {
        if constexpr (sizeof(T) == 8) {
            acc -= partials[(long long)y * N + j];
        } else {
            acc = csub(acc, partials[(long long)y * N + j]);
        }
    }
    return acc;
}

// The new factor row (the updated column times the pivot's scale; the real
// path symmetrises (mu nu) with (nu mu)), the residual update and its
// argmax/minimum.  Each block reduces its entries into partial[block]; the
// last block to finish (counted in st->done) merges the partials in block
// order, as a separate reduction kernel would, ends the step (rank, step
// count) and, unless this is the chain's last step, selects the next pivot.
template <typename T>
__global__ void chain_update_kernel(ChainState* st, const T* pool, const T* partials, int nchunks, int n, T* L,
                                    double* res, Red* partial, Red* out, int* slot_of, long long* log, double tol,
                                    double psd, int select_next) {
    if (!st->active) return;
    const long long N = (long long)n * n;
    const long long piv = st->pivot;
    const T* col_in = pool + (long long)st->slot * N;
    T* Lrow = L + (long long)st->rank * N;
    const double sc = st->scale;
    Red r{-1.0 / 0.0, (long long)1 << 62, 1.0 / 0.0};
    for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < N; j += (long long)gridDim.x * blockDim.x) {
        double mag2;
        if constexpr (sizeof(T) == 8) {
            const long long mu = j / n, nu = j - mu * n;
            const double wj = chain_column(col_in, partials, nchunks, N, j);
            const double wt = chain_column(col_in, partials, nchunks, N, nu * n + mu);
            const double c = (wj + wt) * 0.5 * sc;
            Lrow[j] = c;
            mag2 = c * c;
        } else {
            const double2 c = cscale(chain_column(col_in, partials, nchunks, N, j), sc);
            Lrow[j] = c;
            mag2 = c.x * c.x + c.y * c.y;
        }
        const double nr = res[j] - mag2;
        const double kept = j == piv ? 0.0 : fmax(nr, 0.0);
        res[j] = kept;
        red_merge(r, Red{kept, j, nr});
    }
    r = block_reduce(r);
    __shared__ int last;
    if (threadIdx.x == 0) {
        partial[blockIdx.x] = r;
        __threadfence();
        last = atomicAdd(&st->done, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    Red q{-1.0 / 0.0, (long long)1 << 62, 1.0 / 0.0};
    const volatile Red* vp = partial;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) red_merge(q, Red{vp[i].maxv, vp[i].idx, vp[i].minv});
    q = block_reduce(q);
    if (threadIdx.x == 0) {
        *out = q;
        st->done = 0;
        st->rank += 1;
        st->steps += 1;
        if (select_next) chain_select(st, q, slot_of, log, tol, psd);
    }
}

cudaError_t launch_chol_chain(bool real, void* L, long long N, int n, int rank_hi, int steps, ChainState* st,
                              int* slot_of, long long* log, const void* pool, double* res, void* partial, void* out,
                              void* gemv_partials, int max_chunks, int sms, double tol, double psd, cudaStream_t s) {
    const int blocks = (int)((N + 127) / 128);
    int nchunks = 1;
    if (gemv_partials && max_chunks > 1 && rank_hi >= 64 && sms > 0)
        nchunks = std::max(1, std::min(max_chunks, (8 * sms) / std::max(blocks, 1)));
    const dim3 grid(blocks, nchunks);
    Red* red = static_cast<Red*>(out);
    if (steps > 0) chain_select_kernel<<<1, 1, 0, s>>>(st, red, slot_of, log, tol, psd);
    for (int k = 0; k < steps; ++k) {
        const int select_next = k + 1 < steps ? 1 : 0;
        if (real) {
            chain_gemv_split_kernel<double><<<grid, 128, 0, s>>>(static_cast<const double*>(L), N, st, nchunks,
                                                                 static_cast<double*>(gemv_partials), N);
            chain_update_kernel<double><<<RED_BLOCKS, 256, 0, s>>>(
                st, static_cast<const double*>(pool), static_cast<const double*>(gemv_partials), nchunks, n,
                static_cast<double*>(L), res, static_cast<Red*>(partial), red, slot_of, log, tol, psd, select_next);
        } else {
            chain_gemv_split_kernel<double2><<<grid, 128, 0, s>>>(static_cast<const double2*>(L), N, st, nchunks,
                                                                  static_cast<double2*>(gemv_partials), N);
            chain_update_kernel<double2><<<RED_BLOCKS, 256, 0, s>>>(
                st, static_cast<const double2*>(pool), static_cast<const double2*>(gemv_partials), nchunks, n,
                static_cast<double2*>(L), res, static_cast<Red*>(partial), red, slot_of, log, tol, psd, select_next);
        }
    }
    return cudaGetLastError();
}

// Real factor rows widened to complex128 (imaginary parts zero), for the
// copy to the caller.
__global__ void widen_real_kernel(const double* __restrict__ src, double2* __restrict__ dst, long long n) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        dst[i] = make_double2(src[i], 0.0);
}

cudaError_t launch_widen_real(const double* src, double2* dst, long long n, int sms, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    const int grid = (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 8LL * std::max(sms, 1)));
    widen_real_kernel<<<grid, 256, 0, s>>>(src, dst, n);
    return cudaGetLastError();
}

// residual = D - sum_P |L_P|^2 (used when screened diagonal blocks are measured at the end)
template <typename T>
__global__ void chol_final_residual_kernel(const double* D, const T* L, int rank, long long N, double* res) {
    for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < N; j += (long long)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int r = 0; r < rank; ++r) {
            const T v = L[(long long)r * N + j];
            if constexpr (sizeof(T) == 8)
                s += v * v;
            else
                s += v.x * v.x + v.y * v.y;
        }
        res[j] = D[j] - s;
    }
}

cudaError_t launch_chol_final_residual(bool real, const double* D, const void* L, int rank, long long N, double* res,
                                       cudaStream_t s) {
    const int blocks = (int)((N + 255) / 256);
    if (real)
        chol_final_residual_kernel<double><<<blocks, 256, 0, s>>>(D, static_cast<const double*>(L), rank, N, res);
    else
        chol_final_residual_kernel<double2><<<blocks, 256, 0, s>>>(D, static_cast<const double2*>(L), rank, N, res);
    return cudaGetLastError();
}

size_t chol_red_bytes() { return sizeof(Red); }
size_t chol_partial_bytes() { return sizeof(Red) * RED_BLOCKS; }

}  // namespace gx
