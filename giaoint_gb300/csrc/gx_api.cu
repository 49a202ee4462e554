// Host side of the GB300 electron-repulsion library: the C ABI declared in
// include/giao_gb300.h.  Owns the device context (stream, Boys table, pools),
// uploads bases, builds the per-(basis, field) primitive-pair records, plans
// class-sorted quartet launches and maps device status words to the
// reference's error semantics.
#include <algorithm>
#include <array>
#include <chrono>
#include <limits>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <future>
#include <list>
#include <map>
#include <memory>
#include <mutex>
#include <numeric>
#include <string>
#include <tuple>
#include <unordered_map>
#include <vector>

#include "../../include/giao_gb300.h"
#include "gx_internal.h"

using gx::c2;

namespace {

thread_local std::string g_error;

int fail(int code, const std::string& msg) {
    g_error = msg;
    return code;
}

struct CudaFailure {
    cudaError_t err;
    const char* where;
};

#define GX_CUDA(call)                                    \
    do {                                                 \
        cudaError_t e_ = (call);                         \
        if (e_ != cudaSuccess) throw CudaFailure{e_, #call}; \
    } while (0)

struct ApiError {
    int code;
    std::string msg;
};

[[noreturn]] void raise(int code, const std::string& msg) { throw ApiError{code, msg}; }

template <typename F>
int guarded(F&& f) {
    try {
        f();
        return GX_OK;
    } catch (const ApiError& e) {
        return fail(e.code, e.msg);
    } catch (const CudaFailure& e) {
        return fail(GX_ECUDA, std::string("CUDA error in ") + e.where + ": " + cudaGetErrorString(e.err));
    } catch (const std::bad_alloc&) {
        return fail(GX_ENOMEM, "host allocation failed");
    } catch (const std::exception& e) {
        return fail(GX_EINVAL, e.what());
    }
}

// Grow-only device buffer.
struct DeviceBuffer {
    void* ptr = nullptr;
    size_t bytes = 0;
    void reserve(size_t n) {
        if (n <= bytes) return;
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
        const size_t want = std::max<size_t>(n, 256);
        cudaError_t e = cudaMalloc(&ptr, want);
        if (e != cudaSuccess) {
            cudaGetLastError();
            raise(GX_ENOMEM, "device allocation of " + std::to_string(want) + " bytes failed");
        }
        bytes = want;
    }
    template <typename T>
    T* as() const {
        return static_cast<T*>(ptr);
    }
    void release() {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
    }
    ~DeviceBuffer() { release(); }
};

template <typename T>
void upload(DeviceBuffer& buf, const std::vector<T>& v, cudaStream_t s) {
    buf.reserve(sizeof(T) * std::max<size_t>(v.size(), 1));
    if (!v.empty()) GX_CUDA(cudaMemcpyAsync(buf.ptr, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, s));
}

// ---- host-side normalisation (src/types.cpp:20-72, 136-157) ---------------

double log_odd_double_factorial(int l) {
    if (l == 0) return 0.0;
    const double n = (double)l;
    return n * std::log(2.0) + std::lgamma(n + 0.5) - 0.5 * std::log(M_PI);
}

double primitive_norm(double a, int lx, int ly, int lz) {
    const double total = (double)(lx + ly + lz);
    const double den = log_odd_double_factorial(lx) + log_odd_double_factorial(ly) + log_odd_double_factorial(lz);
    return std::exp(0.75 * std::log(2.0 * a / M_PI) + 0.5 * (total * std::log(4.0 * a) - den));
}

double same_center_overlap(double a, double b, int l) {
    const double norm = primitive_norm(a, l, 0, 0) * primitive_norm(b, l, 0, 0);
    const double p = a + b;
    return norm * std::exp(std::lgamma(l + 0.5) - (l + 0.5) * std::log(p)) * M_PI / p;
}

// Gauss-Legendre nodes (Newton iteration on P_n).
void gauss_legendre(int n, double* x, double* w) {
    for (int i = 0; i < n / 2; ++i) {
        double root = std::cos(M_PI * (i + 0.75) / (n + 0.5));
        double deriv = 0.0;
        for (int it = 0; it < 100; ++it) {
            double p0 = 1.0, p1 = root;
            for (int k = 2; k <= n; ++k) {
                const double p2 = ((2.0 * k - 1.0) * root * p1 - (k - 1.0) * p0) / k;
                p0 = p1;
                p1 = p2;
            }
            deriv = n * (root * p1 - p0) / (root * root - 1.0);
            const double upd = p1 / deriv;
            root -= upd;
            if (std::fabs(upd) < 1e-16) break;
        }
        const double wt = 2.0 / ((1.0 - root * root) * deriv * deriv);
        x[i] = -root;
        x[n - 1 - i] = root;
        w[i] = wt;
        w[n - 1 - i] = wt;
    }
}

// ---- pair classes -----------------------------------------------------------

struct PairClassHost {
    int la, lb, nab, Etot;
    std::vector<int> boxoff, boxdim;
    std::vector<uint32_t> ent;
    DeviceBuffer d_boxoff, d_boxdim, d_ent;
    gx::PairClassDev dev() const {
        return gx::PairClassDev{la, lb, nab, la + lb, Etot, d_boxoff.as<int>(), d_boxdim.as<int>(),
                                d_ent.as<uint32_t>()};
    }
};

std::vector<std::array<int, 3>> components(int l) {
    std::vector<std::array<int, 3>> c;
    for (int x = l; x >= 0; --x)
        for (int y = l - x; y >= 0; --y) c.push_back({x, y, l - x - y});
    return c;
}

}  // namespace

// ---------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------

// Immutable device tables shared by every context on a device: the Boys
// table (132 MB, 93 ms to build), the Gauss-Legendre rules, the Hermite
// index table and the recurrence plans.  Built by the first context on a
// device and kept while any context on it lives.
struct SharedTables {
    DeviceBuffer boys_S, boys_E0, gl, herm, rec_plan, rec_plan_off;
    double boys_table_agreement = 0.0;
};

struct ShapeGraph;  // a column-evaluation CUDA graph (see cholesky_core)
struct ColumnPlan;  // the column-evaluation plan of one pivot shell pair (see cholesky_core)

// Page-locked host memory that grows on demand.
struct PinnedHost {
    void* p = nullptr;
    size_t n = 0;
    PinnedHost() = default;
    PinnedHost(const PinnedHost&) = delete;
    PinnedHost& operator=(const PinnedHost&) = delete;
    ~PinnedHost() {
        if (p) cudaFreeHost(p);
    }
    void reserve(size_t bytes) {
        if (bytes <= n) return;
        if (p) cudaFreeHost(p);
        p = nullptr;
        n = 0;
        GX_CUDA(cudaHostAlloc(&p, bytes, cudaHostAllocDefault));
        n = bytes;
    }
};

struct gx_context {
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t own_stream = nullptr;
    // auxiliary streams on which the class launches of one plan execution run
    // concurrently (fork/join with events on `stream`)
    std::vector<cudaStream_t> aux;
    std::vector<cudaEvent_t> aux_done;
    cudaEvent_t fork = nullptr;
    std::shared_ptr<SharedTables> t;  // shared immutable tables of the device
    DeviceBuffer status;
    std::mutex mu;
    std::map<std::pair<int, int>, std::unique_ptr<PairClassHost>> pair_classes;
    // scratch
    DeviceBuffer out, tasks, scratch_a, scratch_b, scratch_c;
    DeviceBuffer deriv_vals, deriv_meta;
    gx_cholesky_stats last_cholesky{};  // of the last factorisation on this context
    bool stable_launch = false;         // plans built here use size-independent launch configurations
    // page-locked chunk buffers of gx_eri_for_each (held by stream_mu for a
    // whole call)
    PinnedHost stream_host[2];
    std::mutex stream_mu;
    // host-output calls: the output ranges' copies run on copy_stream while
    // later ranges are evaluated; copy_parts = ranges per call (0: by size)
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t copy_done = nullptr;
    int copy_parts = 0;
    // per-class host copies: streams that trail the class streams (so a copy
    // never holds back the next class on its stream) and their join events
    std::vector<cudaStream_t> class_copy;
    std::vector<cudaEvent_t> class_copy_done;
    cudaEvent_t class_done = nullptr;
    // Cholesky column-evaluation graphs by plan shape and device view, kept
    // across factorisations (cleared beyond kMaxShapeGraphs)
    std::map<std::vector<long long>, std::shared_ptr<ShapeGraph>> shape_graphs;
    // page-locked staging of the Cholesky host loop (chain state, reduction,
    // status, chain log; the column-slot map), so its small copies never stall
    PinnedHost chol_mail, chol_slots;
    // Cholesky column plans by (basis, pivot shell pair, real path), kept
    // across factorisations of the same basis (fields change only the pair
    // records); dropped with the basis, cleared beyond kMaxColumnPlanBytes
    std::map<std::tuple<const gx_basis*, int, int, bool>, std::shared_ptr<ColumnPlan>> column_plans;
    size_t column_plan_bytes = 0;
    double copy_first = 0.0;  // share of the output in the first range (0: equal ranges)

    PairClassHost& pair_class(int la, int lb) {
        auto key = std::make_pair(la, lb);
        auto it = pair_classes.find(key);
        if (it != pair_classes.end()) return *it->second;
        auto pc = std::make_unique<PairClassHost>();
        pc->la = la;
        pc->lb = lb;
        const auto ca = components(la), cb = components(lb);
        pc->nab = (int)(ca.size() * cb.size());
        int off = 0;
        for (const auto& a : ca)
            for (const auto& b : cb) {
                const int bx = a[0] + b[0] + 1, by = a[1] + b[1] + 1, bz = a[2] + b[2] + 1;
                pc->boxoff.push_back(off);
                pc->boxdim.push_back(bx | (by << 8) | (bz << 16));
                for (int k = 0; k < bx; ++k)
                    for (int l = 0; l < by; ++l)
                        for (int m = 0; m < bz; ++m) pc->ent.push_back((uint32_t)(k | (l << 8) | (m << 16)));
                off += bx * by * bz;
            }
        pc->Etot = off;
        upload(pc->d_boxoff, pc->boxoff, stream);
        upload(pc->d_boxdim, pc->boxdim, stream);
        upload(pc->d_ent, pc->ent, stream);
        auto& ref = *pc;
        pair_classes.emplace(key, std::move(pc));
        return ref;
    }

    gx::BoysTable boys() const {
        return gx::BoysTable{t->boys_S.as<double2>(), t->boys_E0.as<double2>()};
    }

    void reset_status() { GX_CUDA(cudaMemsetAsync(status.ptr, 0, sizeof(gx::DevStatus), stream)); }

    gx::DevStatus read_status() {
        gx::DevStatus st;
        GX_CUDA(cudaMemcpyAsync(&st, status.ptr, sizeof st, cudaMemcpyDeviceToHost, stream));
        GX_CUDA(cudaStreamSynchronize(stream));
        return st;
    }
};

namespace {

std::string boys_domain_message(double zr, double zi, int order) {
    char buf[320];
    std::snprintf(buf, sizeof buf,
                  "complex Boys argument (%.17g,%.17g) at order %d is outside the verified direct domain |z| <= 160 "
                  "and the conservative large-positive asymptotic sector",
                  zr, zi, order);
    return buf;
}

void check_status(gx_context* ctx) {
    const gx::DevStatus st = ctx->read_status();
    if (st.code == 0) return;
    if (st.code == -4) raise(GX_EBOYS, boys_domain_message(st.zr, st.zi, st.order));
    if (st.code == -40) raise(GX_EBOYS, "requested Boys scaling is not representable for this argument");
    if (st.code == -5) raise(GX_EBOYS, "adaptive complex Boys quadrature did not reach tolerance");
    raise(GX_ECUDA, "device status " + std::to_string(st.code));
}

}  // namespace

// ---------------------------------------------------------------------------
// basis
// ---------------------------------------------------------------------------

struct FieldPairs {
    double B[3], O[3];
    DeviceBuffer p, Pr, Pi, F, Epool, bound, Epool32, order, sbound, g32;
};

struct gx_basis {
    gx_context* ctx = nullptr;
    int ns = 0;
    std::vector<double> center;
    std::vector<int> l, nprim, ncontr;
    std::vector<double> exps, coefs;
    std::vector<int> raw;
    std::vector<int64_t> ao_off;
    int64_t nao = 0;
    // segmented shells: shell s, contraction x -> seg_first[s] + x
    int nseg = 0;
    std::vector<int> seg_first, seg_l, seg_nprim, seg_primoff, seg_raw, seg_orig;
    std::vector<double> seg_center, seg_exps, seg_coefs;
    DeviceBuffer d_center, d_l, d_nprim, d_primoff, d_exps, d_coefs, d_raw, d_sp_off;
    // pair structure (field independent)
    int npp = 0;
    std::vector<int> sp_off, pp_class;
    std::vector<long long> Eoff;
    long long Etotal = 0;
    DeviceBuffer d_pp_a, d_pp_b, d_pp_pa, d_pp_pb, d_pp_class, d_Eoff, d_classes;
    std::vector<std::pair<int, int>> class_keys;
    std::unique_ptr<FieldPairs> pairs;
    // centre-derivative basis (built on first use): the shells of this basis
    // followed by their Z, U and D shells, and per-shell arrays for the
    // combine kernel
    std::unique_ptr<gx_basis> deriv;
    DeviceBuffer d_shell_l, d_shell_ncontr, d_shell_raw, d_shell_center, d_shell_inv2a;
    std::vector<double> shell_inv2a;  // 1 / (2 alpha) of single-primitive shells (l <= 15), else 0
    // derivative-bound basis (built on first use): one raw single-primitive
    // shell per (primitive, variant l / l + 1 / l - 1); bound_index[3 * g + v]
    // for the g-th primitive of the basis (-1: absent)
    std::unique_ptr<gx_basis> bound;
    std::vector<int> bound_index;

    gx::BasisDev dev() const {
        return gx::BasisDev{nseg, d_center.as<double>(), d_l.as<int>(), d_nprim.as<int>(), d_primoff.as<int>(),
                            d_exps.as<double>(), d_coefs.as<double>(), d_raw.as<int>(), d_sp_off.as<int>()};
    }
    int ncart_of(int s) const { return gx::ncart(l[s]); }
    int64_t nao_of(int s) const { return (int64_t)ncontr[s] * ncart_of(s); }
};

namespace {

void build_segments(gx_basis* b) {
    cudaStream_t s = b->ctx->stream;
    b->seg_first.assign(b->ns, 0);
    size_t e = 0, c = 0;
    for (int sh = 0; sh < b->ns; ++sh) {
        b->seg_first[sh] = b->nseg;
        for (int x = 0; x < b->ncontr[sh]; ++x) {
            b->seg_l.push_back(b->l[sh]);
            b->seg_nprim.push_back(b->nprim[sh]);
            b->seg_primoff.push_back((int)b->seg_exps.size());
            b->seg_raw.push_back(b->raw[sh]);
            b->seg_orig.push_back(sh);
            for (int k = 0; k < 3; ++k) b->seg_center.push_back(b->center[3 * sh + k]);
            for (int p = 0; p < b->nprim[sh]; ++p) {
                b->seg_exps.push_back(b->exps[e + p]);
                b->seg_coefs.push_back(b->coefs[c + (size_t)x * b->nprim[sh] + p]);
            }
            ++b->nseg;
        }
        e += b->nprim[sh];
        c += (size_t)b->nprim[sh] * b->ncontr[sh];
    }
    upload(b->d_center, b->seg_center, s);
    upload(b->d_l, b->seg_l, s);
    upload(b->d_nprim, b->seg_nprim, s);
    upload(b->d_primoff, b->seg_primoff, s);
    upload(b->d_exps, b->seg_exps, s);
    upload(b->d_coefs, b->seg_coefs, s);
    upload(b->d_raw, b->seg_raw, s);
    // every ordered segmented shell pair, primitive pairs pa-major
    const int ns = b->nseg;
    std::map<std::pair<int, int>, int> cls;
    std::vector<int> pp_a, pp_b, pp_pa, pp_pb;
    b->sp_off.assign((size_t)ns * ns, 0);
    for (int a = 0; a < ns; ++a)
        for (int bb = 0; bb < ns; ++bb) {
            b->sp_off[(size_t)a * ns + bb] = (int)pp_a.size();
            auto key = std::make_pair(b->seg_l[a], b->seg_l[bb]);
            auto it = cls.find(key);
            int ci;
            if (it == cls.end()) {
                ci = (int)b->class_keys.size();
                cls.emplace(key, ci);
                b->class_keys.push_back(key);
            } else {
                ci = it->second;
            }
            const PairClassHost& pc = b->ctx->pair_class(key.first, key.second);
            for (int pa = 0; pa < b->seg_nprim[a]; ++pa)
                for (int pb = 0; pb < b->seg_nprim[bb]; ++pb) {
                    pp_a.push_back(a);
                    pp_b.push_back(bb);
                    pp_pa.push_back(pa);
                    pp_pb.push_back(pb);
                    b->pp_class.push_back(ci);
                    b->Eoff.push_back(b->Etotal);
                    b->Etotal += pc.Etot;
                }
        }
    b->npp = (int)pp_a.size();
    upload(b->d_sp_off, b->sp_off, s);
    upload(b->d_pp_a, pp_a, s);
    upload(b->d_pp_b, pp_b, s);
    upload(b->d_pp_pa, pp_pa, s);
    upload(b->d_pp_pb, pp_pb, s);
    upload(b->d_pp_class, b->pp_class, s);
    upload(b->d_Eoff, b->Eoff, s);
    std::vector<gx::PairClassDev> devs;
    for (const auto& k : b->class_keys) devs.push_back(b->ctx->pair_class(k.first, k.second).dev());
    upload(b->d_classes, devs, s);
}

// Primitive-pair records for (B, O); cached on the basis for the last field.
// Primitive-pair records for (B, O); cached on the basis for the last field.
// After the records, every primitive pair's exact Schwarz factor is computed
// on the device and each shell pair's primitive pairs are ordered by
// decreasing factor, so that screened primitive quartets form a suffix of
// every bra row and ket column.
gx::PairData pair_view(gx_basis* b, FieldPairs& fp) {
    return gx::PairData{b->npp,
                        fp.p.as<double>(),
                        fp.Pr.as<double>(),
                        fp.Pi.as<double>(),
                        fp.F.as<double2>(),
                        b->d_Eoff.as<long long>(),
                        fp.Epool.as<double2>(),
                        fp.bound.as<double>(),
                        fp.Epool32.as<float2>(),
                        fp.order.as<int>(),
                        fp.sbound.as<float>(),
                        fp.g32.as<float4>()};
}

FieldPairs& field_pairs(gx_basis* b, const double* B, const double* O) {
    if (b->pairs && std::memcmp(b->pairs->B, B, sizeof(double) * 3) == 0 &&
        std::memcmp(b->pairs->O, O, sizeof(double) * 3) == 0)
        return *b->pairs;
    if (!b->pairs) b->pairs = std::make_unique<FieldPairs>();
    FieldPairs& fp = *b->pairs;
    std::memcpy(fp.B, B, sizeof fp.B);
    std::memcpy(fp.O, O, sizeof fp.O);
    const size_t n = std::max(b->npp, 1);
    fp.p.reserve(n * sizeof(double));
    fp.Pr.reserve(3 * n * sizeof(double));
    fp.Pi.reserve(3 * n * sizeof(double));
    fp.F.reserve(n * sizeof(double2));
    fp.bound.reserve(n * sizeof(double));
    fp.order.reserve(n * sizeof(int));
    fp.sbound.reserve(n * sizeof(float));
    fp.g32.reserve(2 * n * sizeof(float4));
    fp.Epool.reserve(std::max<long long>(b->Etotal, 1) * sizeof(double2));
    fp.Epool32.reserve(std::max<long long>(b->Etotal, 1) * sizeof(float2));
    gx::EriDev dev{};
    dev.basis = b->dev();
    dev.pairs = pair_view(b, fp);
    dev.boys = b->ctx->boys();
    dev.gl = b->ctx->t->gl.as<gx::GLRules>();
    dev.herm_xyz = b->ctx->t->herm.as<uint32_t>();
    dev.rec_plan = b->ctx->t->rec_plan.as<int2>();
    dev.rec_plan_off = b->ctx->t->rec_plan_off.as<int>();
    GX_CUDA(gx::launch_pair_precompute(b->dev(), B, O, b->npp, b->d_pp_a.as<int>(), b->d_pp_b.as<int>(),
                                       b->d_pp_pa.as<int>(), b->d_pp_pb.as<int>(), b->d_pp_class.as<int>(),
                                       b->d_classes.as<gx::PairClassDev>(), fp.p.as<double>(), fp.Pr.as<double>(),
                                       fp.Pi.as<double>(), fp.F.as<double2>(), b->d_Eoff.as<long long>(),
                                       fp.Epool.as<double2>(), fp.Epool32.as<float2>(), fp.bound.as<double>(),
                                       fp.g32.as<float4>(), &dev, b->ctx->stream));
    std::vector<double> bound(b->npp);
    if (b->npp)
        GX_CUDA(cudaMemcpyAsync(bound.data(), fp.bound.ptr, b->npp * sizeof(double), cudaMemcpyDeviceToHost,
                                b->ctx->stream));
    GX_CUDA(cudaStreamSynchronize(b->ctx->stream));
    std::vector<int> order(b->npp);
    std::vector<float> sbound(b->npp);
    const int ns = b->nseg;
    for (int a = 0; a < ns; ++a)
        for (int c = 0; c < ns; ++c) {
            const int first = b->sp_off[(size_t)a * ns + c];
            const int count = b->seg_nprim[a] * b->seg_nprim[c];
            std::iota(order.begin() + first, order.begin() + first + count, first);
            std::stable_sort(order.begin() + first, order.begin() + first + count,
                             [&](int x, int y) { return bound[x] > bound[y]; });
            for (int k = first; k < first + count; ++k)
                sbound[k] = (float)std::min(bound[order[k]], 3.0e38);
        }
    upload(fp.order, order, b->ctx->stream);
    upload(fp.sbound, sbound, b->ctx->stream);
    return fp;
}

void check_field(const double* B, const double* O) {
    for (int k = 0; k < 3; ++k) {
        if (!std::isfinite(B[k])) raise(GX_EINVAL, "B values must be finite");
        if (!std::isfinite(O[k])) raise(GX_EINVAL, "gauge_origin values must be finite");
    }
}

// ---- quartet evaluation ------------------------------------------------------

struct QuartetRequest {
    uint32_t a, b, c, d;   // original shells
    int64_t out_off;       // complex-element offset of the block
};

// Class-sorted task list for a set of quartet blocks (field independent).
struct PlanClass {
    std::array<int, 4> key;
    size_t first, count;
    int64_t primitive_quartets;
    double flops_per_primitive_quartet;
};

// Launch configuration of one class: the autotuner's knobs (0 = default).
struct ClassConf {
    int per_group = 0;  // primitive quartets per warp work unit (small: 1024, generic: 32)
    int wpb = 0;        // generic kernel: warps per block cap (4)
    int b1 = 0;         // generic kernel: phase-1 batch cap (32)
    int kt = 0;         // generic kernel: Hermite rows per lane in the ket transform (1, 2, 4; 0 = by lane use)
    int ct = 0;         // generic kernel: ket components per lane in the bra transform (1-4; 0 = by lane use)
    int minb = 0;       // generic kernel: register-budget variant (2 or 4 resident blocks; 0 = 2)
    int nostage = 0;    // generic kernel: 1 = read E~ records and class tables from global memory
    int stream = 0;     // generic kernel: 1 = per-entry recurrences into a two-column buffer (stream mode)
    int nolane = 0;     // 1 = the generic kernel also takes the FP32 entries (no FP32 lane kernel)
};

// Configuration of a class before any tuning, from the autotuner's choices on
// s/p/d molecules in both precision modes and on an s-g atom: two-warp blocks
// for every generic class; below L = 5, 64-primitive-quartet units under the
// four-resident-block register budget (tables read from global memory at
// L = 3); from L = 5 on, stream mode with 16-quartet units, four Hermite
// rows per lane in the ket transform from L = 8, and from L = 12 the
// two-block register budget with phase-1 batches of 16.  Small classes keep
// their own.
ClassConf default_conf(const std::array<int, 4>& k) {
    ClassConf c{};
    if (gx::small_class(k[0], k[1], k[2], k[3])) return c;
    const int L = k[0] + k[1] + k[2] + k[3];
    c.wpb = 2;
    c.minb = 4;
    if (L < 5) {
        c.per_group = 64;
        c.nostage = L == 3 ? 1 : 0;
        return c;
    }
    c.stream = 1;
    c.per_group = 16;
    c.b1 = 32;
    if (L >= 8) c.kt = 4;
    if (L >= 12) {
        c.minb = 2;
        c.b1 = 16;
    }
    return c;
}

// Warp work units of every class: (first task within the class, task count).
struct GroupSet {
    DeviceBuffer dev;
    std::vector<std::pair<size_t, size_t>> range;  // per class: first group, count
    std::vector<std::pair<size_t, size_t>> lane;   // per class: groups of the FP32 lane kernel (count 0: none)
};

struct PlanData {
    DeviceBuffer tasks, counters;
    GroupSet base;                  // default configuration
    std::vector<PlanClass> classes;
    std::vector<int> task_kk;       // per task (class order): Kab << 16 | Kcd, for regrouping
    std::vector<int> task_part;     // per task: its part (request) of a packed plan; empty for one part
    bool stable = false;            // launch configuration independent of the plan's size (see launch_class)
    std::vector<ClassConf> defconf; // per class: the configuration used before any tuning
    std::vector<int> order;         // launch order: largest model work first, so the longest
                                    // classes start before the short ones fill in around them
    int spread_parts = 1;           // one of this many input ranges run back to back: work units are
                                    // sized for the classes of the whole list
    int64_t ntask = 0, primitive_quartets = 0;
    double model_flops = 0.0;
    // autotuned configuration per precision mode (GX_PRECISION_*)
    struct Tuned {
        bool valid = false;
        GroupSet groups;
        std::vector<ClassConf> conf;
    } tuned[3];
};

// FP64 FLOP model per primitive quartet of class (la, lb, lc, ld): the
// reference-structured MD count (one complex FMA per six-index R entry plus
// the cheaper real-by-complex E.R.E ordering, coefficient accumulation and a
// nominal Boys term).
double model_flops(int la, int lb, int lc, int ld) {
    const int Lab = la + lb, Lcd = lc + ld, L = Lab + Lcd;
    auto T = [](int k) { return (double)(k + 1) * (k + 2) / 2.0; };
    double R = 0.0;
    for (int k = 0; k <= Lab; ++k)
        for (int m = 0; m <= Lcd; ++m) R += T(k) * T(m) * (L - k - m + 1);
    const double Nab = gx::herm_count(Lab), Ncd = gx::herm_count(Lcd);
    const double nab = (double)gx::ncart(la) * gx::ncart(lb), ncd = (double)gx::ncart(lc) * gx::ncart(ld);
    const double ere = std::min(4 * Nab * Ncd * ncd + 4 * nab * Nab * ncd, 4 * nab * Nab * Ncd + 4 * nab * Ncd * ncd);
    return 8 * R + ere + 8 * nab * ncd + 8 * (L + 1);
}

// Plans of recent gx_eri_batch calls, per context: a repeated quartet list
// (same basis, same kept quartets after screening) reuses its class-sorted
// task list and work units instead of rebuilding them on the host.  Keyed by
// two independent 64-bit hashes of the kept quartets plus their count and
// output size; at most 4 plans and 2 GiB of task lists per context, least
// recently used first out.  Entries are used with the context's mutex held.
struct CachedPlan {
    const gx_basis* basis;
    uint64_t h1, h2;
    int64_t count, entries;
    int nparts;
    double first_share;
    // the plan of each contiguous input range (one part: the whole list) and
    // the output element at which each part's blocks end
    std::vector<std::unique_ptr<PlanData>> parts;
    std::vector<int64_t> part_end;
};
std::mutex g_plan_cache_mu;
std::map<const gx_context*, std::list<CachedPlan>> g_plan_cache;

std::list<CachedPlan>& plan_cache(const gx_context* ctx) {
    std::lock_guard<std::mutex> lock(g_plan_cache_mu);
    return g_plan_cache[ctx];
}

// Autotuned launch configurations per (context, basis, precision mode) and
// class, recorded by gx_eri_plan_autotune and applied to the plans that
// gx_eri_batch builds for the same basis.
using TuneKey = std::tuple<const gx_context*, const gx_basis*, int>;
std::map<TuneKey, std::map<std::array<int, 4>, ClassConf>> g_tune_db;

// Forget the cached plans and tunings of a basis (null: of the whole context).
void drop_cached_plans(const gx_context* ctx, const gx_basis* b) {
    std::lock_guard<std::mutex> lock(g_plan_cache_mu);
    for (auto it = g_tune_db.begin(); it != g_tune_db.end();) {
        if (std::get<0>(it->first) == ctx && (!b || std::get<1>(it->first) == b))
            it = g_tune_db.erase(it);
        else
            ++it;
    }
    auto it = g_plan_cache.find(ctx);
    if (it == g_plan_cache.end()) return;
    if (!b) {
        g_plan_cache.erase(it);
        return;
    }
    it->second.remove_if([&](const CachedPlan& c) { return c.basis == b; });
}

void record_tuning(const gx_context* ctx, const gx_basis* b, int precision, const PlanData& plan,
                   const std::vector<ClassConf>& conf) {
    std::lock_guard<std::mutex> lock(g_plan_cache_mu);
    auto& db = g_tune_db[TuneKey{ctx, b, precision}];
    for (size_t ci = 0; ci < plan.classes.size(); ++ci) db[plan.classes[ci].key] = conf[ci];
}

// Warp work units of class ci: runs of tasks with equal primitive counts
// (Kab, Kcd).  Small classes (one lane per primitive quartet) take up to
// `per_group` (default 1024) primitive quartets and 128 tasks per unit; the
// generic kernel about `per_group` (default 32) primitive quartets and at
// most 1024 tasks per unit, fewer tasks when the class is too small to give
// every SM eight warps.
std::vector<int2> make_groups(const gx_context* ctx, const PlanData& plan, size_t ci, const ClassConf& conf,
                              bool lane_units = false) {
    const PlanClass& pc = plan.classes[ci];
    const bool small = lane_units || gx::small_class(pc.key[0], pc.key[1], pc.key[2], pc.key[3]);
    const int per = lane_units ? 1024 : (conf.per_group > 0 ? conf.per_group : (small ? 1024 : 32));
    const size_t count = pc.count * (size_t)std::max(plan.spread_parts, 1);
    const int spread = std::max<int>(1, (int)(count / (size_t)(8 * std::max(ctx->sm_count, 1))));
    std::vector<int2> groups;
    size_t i = pc.first;
    const size_t end = pc.first + pc.count;
    while (i < end) {
        const int kk_code = plan.task_kk[i];
        const int kk = (kk_code >> 16) * (kk_code & 0xffff);
        // one lane per primitive quartet: up to `per` of them and 128 tasks per
        // unit, but at least ~4 units per SM when the class is small (a
        // Cholesky column plan holds a few dozen tasks per class); a stable
        // plan keeps its units independent of the class size
        int want = small ? std::max(1, std::min(128, per / kk))
                         : std::max(1, std::min({1024, (per + kk - 1) / kk, spread}));
        if (small && !plan.stable)
            want = std::max(1, std::min<int>(want, (int)(count / (size_t)(4 * std::max(ctx->sm_count, 1)))));
        size_t j = i + 1;
        if (plan.task_part.empty()) {
            while (j < end && (int)(j - i) < want && plan.task_kk[j] == kk_code) ++j;
        } else {
            // a packed plan: units never mix requests, so that every request's
            // units (and its results, bit for bit) are those of its plan alone
            while (j < end && (int)(j - i) < want && plan.task_kk[j] == kk_code &&
                   plan.task_part[j] == plan.task_part[i])
                ++j;
        }
        groups.push_back(make_int2((int)(i - pc.first), (int)(j - i)));
        i = j;
    }
    return groups;
}

bool lane_class(const PlanClass& pc) { return gx::lane32_class(pc.key[0], pc.key[1], pc.key[2], pc.key[3]); }

// Work units of every class, and for the classes with an FP32 lane kernel its
// units (one lane per primitive quartet: up to 1024 primitive quartets and 128
// tasks per warp), in one device array.
void make_group_set(gx_context* ctx, const PlanData& plan, const std::vector<ClassConf>& conf, GroupSet& out) {
    const size_t nc = plan.classes.size();
    std::vector<std::vector<int2>> g(nc), lg(nc);
#pragma omp parallel for schedule(dynamic)
    for (long long ci = 0; ci < (long long)nc; ++ci) {
        g[ci] = make_groups(ctx, plan, ci, conf[ci]);
        if (lane_class(plan.classes[ci])) lg[ci] = make_groups(ctx, plan, ci, conf[ci], true);
    }
    std::vector<int2> all;
    out.range.clear();
    out.lane.clear();
    for (size_t ci = 0; ci < nc; ++ci) {
        out.range.push_back({all.size(), g[ci].size()});
        all.insert(all.end(), g[ci].begin(), g[ci].end());
    }
    for (size_t ci = 0; ci < nc; ++ci) {
        out.lane.push_back({all.size(), lg[ci].size()});
        all.insert(all.end(), lg[ci].begin(), lg[ci].end());
    }
    upload(out.dev, all, ctx->stream);
}

// Give `plan` the recorded tuning of (basis, precision), when there is one.
void apply_recorded_tuning(gx_context* ctx, const gx_basis* b, int precision, PlanData& plan) {
    if (plan.tuned[precision].valid) return;
    std::vector<ClassConf> conf = plan.defconf;
    {
        std::lock_guard<std::mutex> lock(g_plan_cache_mu);
        auto it = g_tune_db.find(TuneKey{ctx, b, precision});
        if (it == g_tune_db.end()) return;
        for (size_t ci = 0; ci < plan.classes.size(); ++ci) {
            auto c = it->second.find(plan.classes[ci].key);
            if (c != it->second.end()) conf[ci] = c->second;
        }
    }
    make_group_set(ctx, plan, conf, plan.tuned[precision].groups);
    plan.tuned[precision].conf = conf;
    plan.tuned[precision].valid = true;
}

// One request of a plan: its basis, its blocks, and where its segmented
// shells, primitive-pair records and output start in the packed numbering
// (all zero for a plan of one basis).
struct PlanPart {
    const gx_basis* b;
    const std::vector<QuartetRequest>* req;
    int seg_base = 0, pair_base = 0;
    int64_t out_base = 0;
};

// Class-sorted task list of the parts' blocks: one task per segmented shell
// quartet (general contractions split), ordered by class (la, lb, lc, ld),
// then by decreasing bra and ket primitive counts, then by part and request
// order -- a parallel counting sort over (class, Kab, Kcd) buckets: per-chunk
// bucket histograms, one prefix over (bucket, chunk), and a scatter pass.
void build_plan_parts(gx_context* ctx, const std::vector<PlanPart>& parts, PlanData& plan) {
    // shell codes: distinct (l, nprim) of the segmented shells of all parts
    std::map<std::pair<int, int>, int> code_of;
    for (const auto& pt : parts)
        for (int s = 0; s < pt.b->nseg; ++s) code_of.emplace(std::make_pair(pt.b->seg_l[s], pt.b->seg_nprim[s]), 0);
    std::vector<std::pair<int, int>> codes;
    for (auto& kv : code_of) {
        kv.second = (int)codes.size();
        codes.push_back(kv.first);
    }
    const int nsc = (int)codes.size();
    std::vector<std::vector<int>> part_code(parts.size());
    for (size_t pi = 0; pi < parts.size(); ++pi) {
        const gx_basis* b = parts[pi].b;
        part_code[pi].resize(b->nseg);
        for (int s = 0; s < b->nseg; ++s) part_code[pi][s] = code_of[{b->seg_l[s], b->seg_nprim[s]}];
    }
    const int64_t ntuple = (int64_t)nsc * nsc * nsc * nsc;
    if (ntuple > (int64_t)1 << 24) raise(GX_EINVAL, "too many distinct (l, primitive count) shells in one plan");
    // buckets: distinct (la, lb, lc, ld, -Kab, -Kcd) in sorted order
    using BKey = std::array<int, 6>;
    std::vector<BKey> tkey(ntuple);
    for (int64_t t = 0; t < ntuple; ++t) {
        const int c0 = (int)(t / ((int64_t)nsc * nsc * nsc)), c1 = (int)(t / ((int64_t)nsc * nsc) % nsc);
        const int c2 = (int)(t / nsc % nsc), c3 = (int)(t % nsc);
        tkey[t] = BKey{codes[c0].first, codes[c1].first, codes[c2].first, codes[c3].first,
                       -codes[c0].second * codes[c1].second, -codes[c2].second * codes[c3].second};
    }
    std::vector<BKey> bkeys(tkey);
    std::sort(bkeys.begin(), bkeys.end());
    bkeys.erase(std::unique(bkeys.begin(), bkeys.end()), bkeys.end());
    const int nb = (int)bkeys.size();
    std::vector<int> bucket_of(ntuple);
    for (int64_t t = 0; t < ntuple; ++t)
        bucket_of[t] = (int)(std::lower_bound(bkeys.begin(), bkeys.end(), tkey[t]) - bkeys.begin());
    // chunks of requests, never across parts: (part, first, end)
    constexpr int64_t kChunk = 1 << 15;
    struct Chunk {
        int part;
        int64_t first, end;
    };
    std::vector<Chunk> chunks;
    for (size_t pi = 0; pi < parts.size(); ++pi) {
        const int64_t n = (int64_t)parts[pi].req->size();
        for (int64_t f = 0; f < n; f += kChunk) chunks.push_back({(int)pi, f, std::min(n, f + kChunk)});
    }
    if (chunks.empty()) chunks.push_back({0, 0, 0});
    const int64_t nchunk = (int64_t)chunks.size();
    std::vector<int64_t> hist((size_t)nchunk * nb, 0);
    // pass 1: bucket histograms per chunk
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < nchunk; ++c) {
        int64_t* h = hist.data() + (size_t)c * nb;
        if (parts.empty()) continue;
        const PlanPart& pt = parts[chunks[c].part];
        const gx_basis* b = pt.b;
        const std::vector<int>& seg_code = part_code[chunks[c].part];
        auto tuple_of = [&](int a, int bb, int cc, int d) {
            return ((int64_t)(seg_code[a] * nsc + seg_code[bb]) * nsc + seg_code[cc]) * nsc + seg_code[d];
        };
        for (int64_t i = chunks[c].first; i < chunks[c].end; ++i) {
            const auto& r = (*pt.req)[i];
            for (int xa = 0; xa < b->ncontr[r.a]; ++xa)
                for (int xb = 0; xb < b->ncontr[r.b]; ++xb)
                    for (int xc = 0; xc < b->ncontr[r.c]; ++xc)
                        for (int xd = 0; xd < b->ncontr[r.d]; ++xd)
                            ++h[bucket_of[tuple_of(b->seg_first[r.a] + xa, b->seg_first[r.b] + xb,
                                                   b->seg_first[r.c] + xc, b->seg_first[r.d] + xd)]];
        }
    }
    // prefix over (bucket, chunk): the first position of each chunk's run
    std::vector<int64_t> btotal(nb, 0);
    int64_t T = 0;
    for (int bk = 0; bk < nb; ++bk)
        for (int64_t c = 0; c < nchunk; ++c) {
            const int64_t n = hist[(size_t)c * nb + bk];
            hist[(size_t)c * nb + bk] = T;
            T += n;
            btotal[bk] += n;
        }
    for (int bk = 0; bk < nb; ++bk)
        if (btotal[bk] && bkeys[bk][0] + bkeys[bk][1] + bkeys[bk][2] + bkeys[bk][3] > 32)
            raise(GX_EINVAL, "electron repulsion supports combined angular order through 32");
    std::unique_ptr<gx::Task[]> all(new gx::Task[std::max<int64_t>(T, 1)]);
    plan.task_kk.resize(T);
    plan.task_part.assign(parts.size() > 1 ? T : 0, 0);
    // pass 2: scatter
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < nchunk; ++c) {
        int64_t* cur = hist.data() + (size_t)c * nb;
        if (parts.empty()) continue;
        const int pidx = chunks[c].part;
        const PlanPart& pt = parts[pidx];
        const gx_basis* b = pt.b;
        const std::vector<int>& seg_code = part_code[pidx];
        auto tuple_of = [&](int a, int bb, int cc, int d) {
            return ((int64_t)(seg_code[a] * nsc + seg_code[bb]) * nsc + seg_code[cc]) * nsc + seg_code[d];
        };
        for (int64_t i = chunks[c].first; i < chunks[c].end; ++i) {
            const auto& r = (*pt.req)[i];
            const int sh[4] = {(int)r.a, (int)r.b, (int)r.c, (int)r.d};
            int64_t N[4];
            int nc[4];
            for (int k = 0; k < 4; ++k) {
                N[k] = b->nao_of(sh[k]);
                nc[k] = b->ncart_of(sh[k]);
            }
            const int st0 = (int)(N[1] * N[2] * N[3]), st1 = (int)(N[2] * N[3]), st2 = (int)N[3];
            for (int xa = 0; xa < b->ncontr[sh[0]]; ++xa)
                for (int xb = 0; xb < b->ncontr[sh[1]]; ++xb)
                    for (int xc = 0; xc < b->ncontr[sh[2]]; ++xc)
                        for (int xd = 0; xd < b->ncontr[sh[3]]; ++xd) {
                            gx::Task t;
                            const int ga = b->seg_first[sh[0]] + xa, gb = b->seg_first[sh[1]] + xb;
                            const int gc = b->seg_first[sh[2]] + xc, gd = b->seg_first[sh[3]] + xd;
                            t.sa = pt.seg_base + ga;
                            t.sb = pt.seg_base + gb;
                            t.sc = pt.seg_base + gc;
                            t.sd = pt.seg_base + gd;
                            t.out_off = pt.out_base + r.out_off + (int64_t)xa * nc[0] * st0 +
                                        (int64_t)xb * nc[1] * st1 + (int64_t)xc * nc[2] * st2 + (int64_t)xd * nc[3];
                            t.st[0] = st0;
                            t.st[1] = st1;
                            t.st[2] = st2;
                            t.st[3] = 1;
                            t.pab = pt.pair_base + b->sp_off[(size_t)ga * b->nseg + gb];
                            t.pcd = pt.pair_base + b->sp_off[(size_t)gc * b->nseg + gd];
                            const int64_t pos = cur[bucket_of[tuple_of(ga, gb, gc, gd)]]++;
                            all[pos] = t;
                            plan.task_kk[pos] = (b->seg_nprim[ga] * b->seg_nprim[gb]) << 16 |
                                                (b->seg_nprim[gc] * b->seg_nprim[gd]);
                            if (!plan.task_part.empty()) plan.task_part[pos] = pidx;
                        }
        }
    }
    // classes: runs of buckets with the same (la, lb, lc, ld)
    plan.classes.clear();
    plan.primitive_quartets = 0;
    plan.model_flops = 0.0;
    size_t first = 0;
    for (int bk = 0; bk < nb;) {
        const std::array<int, 4> key{bkeys[bk][0], bkeys[bk][1], bkeys[bk][2], bkeys[bk][3]};
        size_t count = 0;
        int64_t np = 0;
        int e = bk;
        for (; e < nb && bkeys[e][0] == key[0] && bkeys[e][1] == key[1] && bkeys[e][2] == key[2] &&
               bkeys[e][3] == key[3];
             ++e) {
            count += btotal[e];
            np += btotal[e] * (int64_t)bkeys[e][4] * bkeys[e][5];  // (-Kab)(-Kcd)
        }
        if (count) {
            const double fl = model_flops(key[0], key[1], key[2], key[3]);
            plan.classes.push_back({key, first, count, np, fl});
            plan.primitive_quartets += np;
            plan.model_flops += (double)np * fl;
            first += count;
        }
        bk = e;
    }
    plan.ntask = T;
    plan.stable = ctx->stable_launch;
    plan.tasks.reserve(sizeof(gx::Task) * std::max<int64_t>(T, 1));
    if (T) GX_CUDA(cudaMemcpyAsync(plan.tasks.ptr, all.get(), sizeof(gx::Task) * T, cudaMemcpyHostToDevice, ctx->stream));
    plan.defconf.resize(plan.classes.size());
    for (size_t ci = 0; ci < plan.classes.size(); ++ci) plan.defconf[ci] = default_conf(plan.classes[ci].key);
    plan.order.resize(plan.classes.size());
    std::iota(plan.order.begin(), plan.order.end(), 0);
    std::stable_sort(plan.order.begin(), plan.order.end(), [&](int x, int y) {
        const PlanClass &a = plan.classes[x], &c = plan.classes[y];
        return (double)a.primitive_quartets * a.flops_per_primitive_quartet >
               (double)c.primitive_quartets * c.flops_per_primitive_quartet;
    });
    make_group_set(ctx, plan, plan.defconf, plan.base);
    // (a copy from pageable memory is staged before cudaMemcpyAsync returns,
    // so the host task array may be freed now)
}

void build_plan(gx_context* ctx, gx_basis* b, const std::vector<QuartetRequest>& req, PlanData& plan) {
    build_plan_parts(ctx, {PlanPart{b, &req}}, plan);
}

// Primitive screening thresholds on the Schwarz product B_P B_Q.  FP64: a
// skipped primitive quartet contributes below 1e-18 to every element, so a
// shell quartet (at most a few thousand primitive quartets) moves by less
// than 1e-14 absolute.  Mixed: 1e-15, with FP32 up to the caller's cutoff.
constexpr double kSkipFP64 = 1e-18;
constexpr double kSkipMixed = 1e-15;

// Device view of one evaluation: pair records for (B, O), thresholds of the
// precision mode, output and counters.
gx::EriDev make_dev(gx_context* ctx, gx_basis* b, FieldPairs& fp, double2* out, int precision, double mixed_cutoff) {
    gx::EriDev dev{};
    const bool mixed = precision == GX_PRECISION_MIXED;
    dev.skip_cut = (float)(mixed ? kSkipMixed : (precision == GX_PRECISION_FP64_EXACT ? 0.0 : kSkipFP64));
    dev.fp32_cut = (float)(mixed ? std::max(mixed_cutoff, kSkipMixed) : 0.0);
    dev.basis = b->dev();
    dev.pairs = pair_view(b, fp);
    dev.boys = ctx->boys();
    dev.gl = ctx->t->gl.as<gx::GLRules>();
    dev.herm_xyz = ctx->t->herm.as<uint32_t>();
    dev.rec_plan = ctx->t->rec_plan.as<int2>();
    dev.rec_plan_off = ctx->t->rec_plan_off.as<int>();
    dev.out = out;
    dev.status = ctx->status.as<gx::DevStatus>();
    return dev;
}

// Enqueue the kernel of class ci with configuration conf and work units
// groups[0..ngroup).  Returns the (batch, warps per block) used through the
// optional pointers.
void launch_class(gx_context* ctx, gx::EriDev dev, const PlanData& plan, size_t ci, const ClassConf& conf,
                  const int2* groups, int ngroup, unsigned long long* counters, cudaStream_t s, int* used_b1 = nullptr,
                  int* used_wpb = nullptr, int* used_tiles = nullptr, const int2* lane_groups = nullptr,
                  int nlane = 0) {
    const auto& pc = plan.classes[ci];
    const auto& k = pc.key;
    dev.counters = counters ? counters + 2 * ci : nullptr;
    if (gx::small_class(k[0], k[1], k[2], k[3])) {
        gx::QuartetClass qc{};
        qc.L = k[0] + k[1] + k[2] + k[3];
        qc.ntask = (int)pc.count;
        qc.tasks = plan.tasks.as<gx::Task>() + pc.first;
        qc.ngroup = ngroup;
        qc.groups = groups;
        GX_CUDA(gx::launch_small(k[0], k[1], k[2], k[3], dev, qc, s));
        if (used_b1) *used_b1 = 32;
        if (used_wpb) *used_wpb = 4;
        return;
    }
    gx::QuartetClass qc{};
    qc.bra = ctx->pair_class(k[0], k[1]).dev();
    qc.ket = ctx->pair_class(k[2], k[3]).dev();
    qc.L = k[0] + k[1] + k[2] + k[3];
    qc.Nab = gx::herm_count(k[0] + k[1]);
    qc.NL = gx::herm_count(qc.L);
    const int ncd = qc.ket.nab;
    qc.CH = std::max(1, std::min(ncd, 2048 / qc.Nab));
    // Few work units: split the ket components of a group over several
    // warps (each chunk keeps at least 32 ket-transform rows per warp).
    // (not in a stable plan: there the configuration of a class does not depend
    // on how many tasks it holds, so a request gives the same bits in any pack)
    const int target_units = 8 * std::max(ctx->sm_count, 1);
    if (!plan.stable && ngroup > 0 && ngroup * ((ncd + qc.CH - 1) / qc.CH) < target_units) {
        const int want = (target_units + ngroup - 1) / ngroup;
        const int ch = std::max((ncd + want - 1) / want, (32 + qc.Nab - 1) / qc.Nab);
        qc.CH = std::max(1, std::min(qc.CH, ch));
    }
    // Lane utilisation of a transform with `items` work items per warp.
    auto util = [](long long items) { return (double)items / (32.0 * (double)((items + 31) / 32)); };
    // Tiles: rows per lane KT of the ket transform and ket components per lane
    // CT of the bra transform, chosen for the best lane utilisation (padding
    // of Nab to a multiple of KT counts as waste), the wider tile on ties.
    if (conf.kt == 1 || conf.kt == 2 || conf.kt == 4) {
        qc.KT = conf.kt;
    } else {
        double best = -1.0;
        for (int kt : {4, 2, 1}) {
            const int nkb = (qc.Nab + kt - 1) / kt;
            const double e = util((long long)nkb * std::min(qc.CH, ncd)) * qc.Nab / (double)(nkb * kt);
            if (e > best * 1.05) {
                best = e;
                qc.KT = kt;
            }
        }
    }
    if (conf.ct >= 1 && conf.ct <= 4 && ncd % conf.ct == 0) {
        qc.CT = conf.ct;
    } else {
        double best = -1.0;
        qc.CT = 1;
        for (int ct : {4, 3, 2, 1}) {
            if (ncd % ct) continue;
            int ch = qc.CH < ncd ? std::max(ct, qc.CH / ct * ct) : ncd;
            const double e = util((long long)qc.bra.nab * (std::min(ch, ncd) / ct));
            if (e > best * 1.05) {
                best = e;
                qc.CT = ct;
            }
        }
    }
    if (qc.CH < ncd) qc.CH = std::max(qc.CT, qc.CH / qc.CT * qc.CT);  // chunks hold whole CT tiles
    qc.nchunk = (ncd + qc.CH - 1) / qc.CH;
    qc.stream = conf.stream ? 1 : 0;
    int B1 = conf.b1 > 0 ? std::min(32, conf.b1) : 32;
    if (qc.stream)
        while (B1 > 1 && (size_t)qc.NL * 2 + (size_t)B1 * (qc.L + 4) + (size_t)qc.Nab * qc.CH > 3584) B1 /= 2;
    else
        while (B1 > 1 && (size_t)qc.NL * (B1 + 1) + (size_t)qc.Nab * qc.CH > 3584) B1 /= 2;
    qc.B1 = B1;
    {
        // cooperative recurrence when a batch has fewer entries than the
        // ratio of the lane-parallel to the cooperative instruction count
        double lane_cost = 150.0, coop_cost = 180.0;
        for (int n = 0; n < qc.L; ++n) {
            const int h = gx::herm_count(qc.L - n);
            lane_cost += 6.0 * (h - 1);
            coop_cost += 10.0 * ((h + 31) / 32);
        }
        qc.coop = std::min(B1, (int)(lane_cost / coop_cost));
    }
    qc.ntask = (int)pc.count;
    qc.tasks = plan.tasks.as<gx::Task>() + pc.first;
    qc.ngroup = ngroup;
    qc.groups = groups;
    qc.minb = conf.minb == 4 ? 4 : 2;
    // stage E~ records per warp and the class tables per block when small
    {
        const int emax = std::max(qc.ket.Etot, qc.bra.Etot);
        qc.stage_e = emax <= 384 && !conf.nostage ? emax : 0;
        const int words = 2 * qc.ket.nab + qc.ket.Etot + 2 * qc.bra.nab + qc.bra.Etot +
                          qc.Nab * gx::herm_count(k[2] + k[3]);
        qc.tab_words = words <= 4096 && !conf.nostage ? words : 0;
    }
    const size_t per_warp = gx::quartet_smem_bytes(qc, 1, dev.fp32_cut > 0.0f);
    const int cap = conf.wpb > 0 ? std::min(4, conf.wpb) : 4;
    const int wpb = (int)std::max<size_t>(1, std::min<size_t>(cap, (200 * 1024) / per_warp));
    const int grid = (int)std::min<long long>(((long long)qc.ngroup * qc.nchunk + wpb - 1) / wpb, 1 << 30);
    // mixed precision: the FP32 entries of a 3 <= L <= 4 class go to the FP32
    // lane kernel, launched after this one on the same stream
    const bool lane = dev.fp32_cut > 0.0f && lane_groups && nlane > 0 && !conf.nolane &&
                      gx::lane32_class(k[0], k[1], k[2], k[3]);
    qc.no32 = lane ? 1 : 0;
    GX_CUDA(gx::launch_quartets(dev, qc, wpb, grid, s));
    if (lane) {
        gx::QuartetClass lq{};
        lq.L = qc.L;
        lq.ntask = qc.ntask;
        lq.tasks = qc.tasks;
        lq.ngroup = nlane;
        lq.groups = lane_groups;
        GX_CUDA(gx::launch_lane32(k[0], k[1], k[2], k[3], dev, lq, s));
    }
    if (used_b1) *used_b1 = B1;
    if (used_wpb) *used_wpb = wpb;
    if (used_tiles) {
        used_tiles[0] = qc.KT;
        used_tiles[1] = qc.CT;
        used_tiles[2] = qc.minb;
    }
}

// Enqueue the pair records for (B, O) and every class launch; no host sync
// unless the field changed (the pair bounds are sorted on the host).  Uses
// the autotuned configuration of the precision mode when there is one.
// counters: 2 per class (FP64, FP32 primitive quartets evaluated) or null;
// zeroed first unless `accumulate`.
// host_mapped (may be null): page-locked host output, its mapped address;
// each class's blocks are copied there by the SMs right after the class.
int enqueue_plan(gx_context* ctx, const gx::EriDev& dev, const PlanData& plan, int precision,
                 unsigned long long* counters, bool accumulate, void* host_mapped = nullptr);

int execute_plan(gx_context* ctx, gx_basis* b, const double* B, const double* O, const PlanData& plan,
                 double2* out, int precision = GX_PRECISION_FP64, double mixed_cutoff = 0.0,
                 unsigned long long* counters = nullptr, bool accumulate = false, void* host_mapped = nullptr) {
    FieldPairs& fp = field_pairs(b, B, O);
    const gx::EriDev dev = make_dev(ctx, b, fp, out, precision, mixed_cutoff);
    return enqueue_plan(ctx, dev, plan, precision, counters, accumulate, host_mapped);
}

// Enqueue every class launch of `plan` for the evaluation view `dev`.
int enqueue_plan(gx_context* ctx, const gx::EriDev& dev, const PlanData& plan, int precision,
                 unsigned long long* counters, bool accumulate, void* host_mapped) {
    cudaStream_t s = ctx->stream;
    // host copies on streams of their own, each waiting for its class (a
    // waited event stands for its latest record, so one event serves all)
    constexpr int kCopyStreams = 8;
    if (host_mapped && ctx->class_copy.empty()) {
        ctx->class_copy.resize(kCopyStreams);
        ctx->class_copy_done.resize(kCopyStreams);
        for (int k = 0; k < kCopyStreams; ++k) {
            GX_CUDA(cudaStreamCreateWithFlags(&ctx->class_copy[k], cudaStreamNonBlocking));
            GX_CUDA(cudaEventCreateWithFlags(&ctx->class_copy_done[k], cudaEventDisableTiming));
        }
        GX_CUDA(cudaEventCreateWithFlags(&ctx->class_done, cudaEventDisableTiming));
    }
    int ncopies = 0;
    auto copy_class = [&](size_t ci, cudaStream_t cs) {
        if (!host_mapped) return;
        const PlanClass& pc = plan.classes[ci];
        cudaStream_t cp = ctx->class_copy[ncopies++ % kCopyStreams];
        GX_CUDA(cudaEventRecord(ctx->class_done, cs));
        GX_CUDA(cudaStreamWaitEvent(cp, ctx->class_done, 0));
        GX_CUDA(gx::launch_class_copy(plan.tasks.as<gx::Task>() + pc.first, (int)pc.count, pc.key[0], pc.key[1],
                                      pc.key[2], pc.key[3], dev.out, host_mapped, ctx->sm_count, cp));
    };
    auto join_copies = [&] {
        if (!host_mapped) return;
        for (int k = 0; k < std::min(ncopies, kCopyStreams); ++k) {
            GX_CUDA(cudaEventRecord(ctx->class_copy_done[k], ctx->class_copy[k]));
            GX_CUDA(cudaStreamWaitEvent(s, ctx->class_copy_done[k], 0));
        }
    };
    if (counters && !accumulate) GX_CUDA(cudaMemsetAsync(counters, 0, 2 * plan.classes.size() * sizeof(unsigned long long), s));
    ctx->reset_status();
    const auto& tuned = plan.tuned[precision];
    const GroupSet& gs = tuned.valid ? tuned.groups : plan.base;
    const size_t nc = plan.classes.size();
    // The classes write disjoint output blocks, so they run concurrently on
    // the auxiliary streams: a plan of many small classes (a Cholesky column
    // batch) costs about its longest class instead of the sum, and the tails
    // of large classes overlap.  Under stream capture this becomes parallel
    // graph branches.
    constexpr int kAux = 32;
    const int K = (int)std::min<size_t>(nc, kAux);
    if (K > 1) {
        if (ctx->aux.empty()) {
            ctx->aux.resize(kAux);
            ctx->aux_done.resize(kAux);
            for (int k = 0; k < kAux; ++k) {
                GX_CUDA(cudaStreamCreateWithFlags(&ctx->aux[k], cudaStreamNonBlocking));
                GX_CUDA(cudaEventCreateWithFlags(&ctx->aux_done[k], cudaEventDisableTiming));
            }
            GX_CUDA(cudaEventCreateWithFlags(&ctx->fork, cudaEventDisableTiming));
        }
        GX_CUDA(cudaEventRecord(ctx->fork, s));
        for (int k = 0; k < K; ++k) GX_CUDA(cudaStreamWaitEvent(ctx->aux[k], ctx->fork, 0));
        for (size_t oi = 0; oi < nc; ++oi) {
            const size_t ci = plan.order.empty() ? oi : (size_t)plan.order[oi];
            launch_class(ctx, dev, plan, ci, tuned.valid ? tuned.conf[ci] : plan.defconf[ci],
                         gs.dev.as<int2>() + gs.range[ci].first, (int)gs.range[ci].second, counters,
                         ctx->aux[oi % K], nullptr, nullptr, nullptr, gs.dev.as<int2>() + gs.lane[ci].first,
                         (int)gs.lane[ci].second);
            copy_class(ci, ctx->aux[oi % K]);
        }
        for (int k = 0; k < K; ++k) {
            GX_CUDA(cudaEventRecord(ctx->aux_done[k], ctx->aux[k]));
            GX_CUDA(cudaStreamWaitEvent(s, ctx->aux_done[k], 0));
        }
        join_copies();
    } else {
        for (size_t ci = 0; ci < nc; ++ci) {
            launch_class(ctx, dev, plan, ci, tuned.valid ? tuned.conf[ci] : plan.defconf[ci],
                         gs.dev.as<int2>() + gs.range[ci].first, (int)gs.range[ci].second, counters, s, nullptr,
                         nullptr, nullptr, gs.dev.as<int2>() + gs.lane[ci].first, (int)gs.lane[ci].second);
            copy_class(ci, s);
        }
        join_copies();
    }
    return 1 + (int)nc;
}

// Enqueue several plans (each with its own evaluation view and counters,
// accumulated) under one fork/join over the auxiliary streams, their class
// launches interleaved round robin.
void enqueue_plans(gx_context* ctx, const std::vector<std::pair<const PlanData*, gx::EriDev>>& runs, int precision,
                   const std::vector<unsigned long long*>& counters) {
    cudaStream_t s = ctx->stream;
    ctx->reset_status();
    constexpr int kAux = 32;
    if (ctx->aux.empty()) {
        ctx->aux.resize(kAux);
        ctx->aux_done.resize(kAux);
        for (int k = 0; k < kAux; ++k) {
            GX_CUDA(cudaStreamCreateWithFlags(&ctx->aux[k], cudaStreamNonBlocking));
            GX_CUDA(cudaEventCreateWithFlags(&ctx->aux_done[k], cudaEventDisableTiming));
        }
        GX_CUDA(cudaEventCreateWithFlags(&ctx->fork, cudaEventDisableTiming));
    }
    GX_CUDA(cudaEventRecord(ctx->fork, s));
    for (int k = 0; k < kAux; ++k) GX_CUDA(cudaStreamWaitEvent(ctx->aux[k], ctx->fork, 0));
    int next = 0;
    for (size_t r = 0; r < runs.size(); ++r) {
        const PlanData& plan = *runs[r].first;
        const auto& tuned = plan.tuned[precision];
        const GroupSet& gs = tuned.valid ? tuned.groups : plan.base;
        for (size_t oi = 0; oi < plan.classes.size(); ++oi, ++next) {
            const size_t ci = plan.order.empty() ? oi : (size_t)plan.order[oi];
            launch_class(ctx, runs[r].second, plan, ci, tuned.valid ? tuned.conf[ci] : plan.defconf[ci],
                         gs.dev.as<int2>() + gs.range[ci].first, (int)gs.range[ci].second, counters[r],
                         ctx->aux[next % kAux], nullptr, nullptr, nullptr, gs.dev.as<int2>() + gs.lane[ci].first,
                         (int)gs.lane[ci].second);
        }
    }
    for (int k = 0; k < kAux; ++k) {
        GX_CUDA(cudaEventRecord(ctx->aux_done[k], ctx->aux[k]));
        GX_CUDA(cudaStreamWaitEvent(s, ctx->aux_done[k], 0));
    }
}

// Blocks of the SM copy to page-locked host memory: a few dozen saturate the
// host link; the rest of the GPU keeps evaluating.
constexpr int kHostCopyBlocks = 64;

// Enqueue the parts of a split plan and, behind each part, the copy of its
// output range to host memory `host` on the context's copy stream (by the SMs
// through `host_mapped` when that is given, else by the copy engine): the
// class launches of later parts keep the SMs busy while earlier ranges are
// copied.
// There is no join between parts; the copy of part r waits until every
// auxiliary stream has finished its launches of parts 0..r.  `compute_done`
// is recorded on the context stream once every class launch has finished;
// the context stream then also waits for the last copy.
void enqueue_parts_with_copies(gx_context* ctx, const gx::EriDev& dev, const CachedPlan& cp, int precision,
                               const std::vector<unsigned long long*>& counters, const double2* dout, void* host,
                               void* host_mapped, cudaEvent_t compute_done) {
    cudaStream_t s = ctx->stream;
    constexpr int kAux = 32;
    if (ctx->aux.empty()) {
        ctx->aux.resize(kAux);
        ctx->aux_done.resize(kAux);
        for (int k = 0; k < kAux; ++k) {
            GX_CUDA(cudaStreamCreateWithFlags(&ctx->aux[k], cudaStreamNonBlocking));
            GX_CUDA(cudaEventCreateWithFlags(&ctx->aux_done[k], cudaEventDisableTiming));
        }
        GX_CUDA(cudaEventCreateWithFlags(&ctx->fork, cudaEventDisableTiming));
    }
    if (!ctx->copy_stream) {
        GX_CUDA(cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
        GX_CUDA(cudaEventCreateWithFlags(&ctx->copy_done, cudaEventDisableTiming));
    }
    for (size_t r = 0; r < cp.parts.size(); ++r)
        if (counters[r])
            GX_CUDA(cudaMemsetAsync(counters[r], 0, 2 * cp.parts[r]->classes.size() * sizeof(unsigned long long), s));
    ctx->reset_status();
    GX_CUDA(cudaEventRecord(ctx->fork, s));
    for (int k = 0; k < kAux; ++k) GX_CUDA(cudaStreamWaitEvent(ctx->aux[k], ctx->fork, 0));
    GX_CUDA(cudaStreamWaitEvent(ctx->copy_stream, ctx->fork, 0));
    int next = 0;
    int64_t start = 0;
    for (size_t r = 0; r < cp.parts.size(); ++r) {
        const PlanData& plan = *cp.parts[r];
        const auto& tuned = plan.tuned[precision];
        const GroupSet& gs = tuned.valid ? tuned.groups : plan.base;
        for (size_t oi = 0; oi < plan.classes.size(); ++oi, ++next) {
            const size_t ci = plan.order.empty() ? oi : (size_t)plan.order[oi];
            launch_class(ctx, dev, plan, ci, tuned.valid ? tuned.conf[ci] : plan.defconf[ci],
                         gs.dev.as<int2>() + gs.range[ci].first, (int)gs.range[ci].second, counters[r],
                         ctx->aux[next % kAux], nullptr, nullptr, nullptr, gs.dev.as<int2>() + gs.lane[ci].first,
                         (int)gs.lane[ci].second);
        }
        // a waited event stands for its latest record, so the events are reused per part
        for (int k = 0; k < kAux; ++k) {
            GX_CUDA(cudaEventRecord(ctx->aux_done[k], ctx->aux[k]));
            GX_CUDA(cudaStreamWaitEvent(ctx->copy_stream, ctx->aux_done[k], 0));
        }
        const int64_t end = cp.part_end[r];
        if (end > start) {
            const int64_t bytes = (end - start) * (int64_t)sizeof(double2);
            if (host_mapped)
                GX_CUDA(gx::launch_host_copy(static_cast<char*>(host_mapped) + start * sizeof(double2), dout + start,
                                             bytes, kHostCopyBlocks, ctx->copy_stream));
            else
                GX_CUDA(cudaMemcpyAsync(static_cast<char*>(host) + start * sizeof(double2), dout + start, bytes,
                                        cudaMemcpyDeviceToHost, ctx->copy_stream));
        }
        start = end;
    }
    for (int k = 0; k < kAux; ++k) GX_CUDA(cudaStreamWaitEvent(s, ctx->aux_done[k], 0));
    GX_CUDA(cudaEventRecord(compute_done, s));
    GX_CUDA(cudaEventRecord(ctx->copy_done, ctx->copy_stream));
    GX_CUDA(cudaStreamWaitEvent(s, ctx->copy_done, 0));
}

// Evaluate blocks of `req` into device buffer `out` (packed, C order, AO
// index = contraction * ncart + component) and wait for them.
void run_plan(gx_context* ctx, gx_basis* b, const double* B, const double* O, PlanData& plan, double2* out,
              float* kernel_ms, int64_t* primitive_quartets, int precision, double mixed_cutoff, int64_t* evaluated);

void run_quartets(gx_context* ctx, gx_basis* b, const double* B, const double* O,
                  const std::vector<QuartetRequest>& req, double2* out, float* kernel_ms,
                  int64_t* primitive_quartets = nullptr, int precision = GX_PRECISION_FP64,
                  double mixed_cutoff = 0.0, int64_t* evaluated = nullptr) {
    PlanData plan;
    build_plan(ctx, b, req, plan);
    run_plan(ctx, b, B, O, plan, out, kernel_ms, primitive_quartets, precision, mixed_cutoff, evaluated);
}

// Evaluate a built plan into `out` and wait for it.
void run_plan(gx_context* ctx, gx_basis* b, const double* B, const double* O, PlanData& plan, double2* out,
              float* kernel_ms, int64_t* primitive_quartets, int precision, double mixed_cutoff, int64_t* evaluated) {
    cudaStream_t s = ctx->stream;
    if (primitive_quartets) *primitive_quartets = plan.primitive_quartets;
    unsigned long long* counters = nullptr;
    if (evaluated) {
        plan.counters.reserve(std::max<size_t>(2 * plan.classes.size(), 2) * sizeof(unsigned long long));
        counters = plan.counters.as<unsigned long long>();
    }
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (kernel_ms) {
        GX_CUDA(cudaEventCreate(&e0));
        GX_CUDA(cudaEventCreate(&e1));
        GX_CUDA(cudaEventRecord(e0, s));
    }
    execute_plan(ctx, b, B, O, plan, out, precision, mixed_cutoff, counters);
    if (kernel_ms) {
        GX_CUDA(cudaEventRecord(e1, s));
        GX_CUDA(cudaEventSynchronize(e1));
        GX_CUDA(cudaEventElapsedTime(kernel_ms, e0, e1));
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
    }
    check_status(ctx);
    if (evaluated) {
        std::vector<unsigned long long> c(2 * plan.classes.size());
        if (!c.empty())
            GX_CUDA(cudaMemcpy(c.data(), counters, c.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
        evaluated[0] = evaluated[1] = 0;
        for (size_t i = 0; i < plan.classes.size(); ++i) {
            evaluated[0] += (int64_t)c[2 * i];
            evaluated[1] += (int64_t)c[2 * i + 1];
        }
    }
}

void validate_quartets(const gx_basis* b, const uint32_t* q, int64_t nq) {
    const uint32_t ns = (uint32_t)b->ns;
    int bad = 0;
#pragma omp parallel for reduction(| : bad) schedule(static)
    for (int64_t i = 0; i < 4 * nq; ++i) bad |= q[i] >= ns;
    if (bad) raise(GX_ERANGE, "ERI shell-quartet index is out of range");
}

std::vector<double> schwarz_values(gx_context* ctx, gx_basis* b, const double* B, const double* O) {
    // (ab|ba) blocks for a <= b, then Q_ab = nextafter(sqrt(max |(ij|ji)|)(1 + 64 eps))
    std::vector<QuartetRequest> req;
    int64_t off = 0;
    for (int a = 0; a < b->ns; ++a)
        for (int c = a; c < b->ns; ++c) {
            req.push_back({(uint32_t)a, (uint32_t)c, (uint32_t)c, (uint32_t)a, off});
            off += b->nao_of(a) * b->nao_of(c) * b->nao_of(c) * b->nao_of(a);
        }
    ctx->scratch_a.reserve(std::max<int64_t>(off, 1) * sizeof(double2));
    // bounds must not lose the tiniest pairs: no primitive screening here
    run_quartets(ctx, b, B, O, req, ctx->scratch_a.as<double2>(), nullptr, nullptr, GX_PRECISION_FP64_EXACT);
    std::vector<std::complex<double>> host(off);
    if (off) GX_CUDA(cudaMemcpy(host.data(), ctx->scratch_a.ptr, off * sizeof(double2), cudaMemcpyDeviceToHost));
    std::vector<double> q((size_t)b->ns * b->ns, 0.0);
    size_t r = 0;
    for (int a = 0; a < b->ns; ++a)
        for (int c = a; c < b->ns; ++c, ++r) {
            const int64_t na = b->nao_of(a), nb = b->nao_of(c);
            const std::complex<double>* blk = host.data() + req[r].out_off;
            double m = 0.0;
            for (int64_t i = 0; i < na; ++i)
                for (int64_t j = 0; j < nb; ++j) m = std::max(m, std::abs(blk[((i * nb + j) * nb + j) * na + i]));
            const double v = std::nextafter(std::sqrt(m) * (1.0 + 64.0 * 2.220446049250313e-16), INFINITY);
            q[(size_t)a * b->ns + c] = v;
            q[(size_t)c * b->ns + a] = v;
        }
    return q;
}

// Upload a basis (caller holds ctx->mu).
std::unique_ptr<gx_basis> new_basis(gx_context* ctx, int nshell, const double* centers, const int* l,
                                    const int* nprim, const int* ncontr, const double* exponents,
                                    const double* coefs, const int* raw) {
    auto b = std::make_unique<gx_basis>();
    b->ctx = ctx;
    b->ns = nshell;
    b->center.assign(centers, centers + 3 * (size_t)nshell);
    b->l.assign(l, l + nshell);
    b->nprim.assign(nprim, nprim + nshell);
    b->ncontr.assign(ncontr, ncontr + nshell);
    size_t ne = 0, nc = 0;
    for (int s = 0; s < nshell; ++s) {
        if (l[s] < 0 || l[s] > 16) raise(GX_EINVAL, "shell angular momentum above 16 is not supported");
        if (nprim[s] <= 0 || ncontr[s] <= 0) raise(GX_EINVAL, "a shell requires primitives and contractions");
        ne += nprim[s];
        nc += (size_t)nprim[s] * ncontr[s];
    }
    b->exps.assign(exponents, exponents + ne);
    b->coefs.assign(coefs, coefs + nc);
    b->raw.assign(nshell, 0);
    if (raw)
        for (int s = 0; s < nshell; ++s) b->raw[s] = raw[s] ? 1 : 0;
    int64_t a = 0;
    for (int s = 0; s < nshell; ++s) {
        b->ao_off.push_back(a);
        a += b->nao_of(s);
    }
    b->nao = a;
    build_segments(b.get());
    GX_CUDA(cudaStreamSynchronize(ctx->stream));
    return b;
}

// Cached plan of basis `b` for a request list identified by (h1, h2, count,
// entries), split into up to `nparts` contiguous input ranges of about equal
// output size (empty ranges dropped); `make()` returns the request list
// (increasing output offsets) on a miss.
template <class Make>
CachedPlan& lookup_parts(gx_context* ctx, gx_basis* b, uint64_t h1, uint64_t h2, int64_t count, int64_t entries,
                         int nparts, Make&& make, double first_share = 0.0, CachedPlan* transient = nullptr) {
    auto& cache = plan_cache(ctx);
    auto hit = std::find_if(cache.begin(), cache.end(), [&](const CachedPlan& c) {
        return c.basis == b && c.h1 == h1 && c.h2 == h2 && c.count == count && c.entries == entries &&
               c.nparts == nparts && c.first_share == first_share;
    });
    if (hit == cache.end() && transient) {
        // built for this call only (the cache keeps the lists that recur)
        const std::vector<QuartetRequest> req = make();
        *transient = CachedPlan{b, h1, h2, count, entries, 1, 0.0, {}, {}};
        transient->parts.push_back(std::make_unique<PlanData>());
        build_plan(ctx, b, req, *transient->parts[0]);
        transient->part_end.push_back(entries);
        return *transient;
    }
    if (hit == cache.end()) {
        const std::vector<QuartetRequest> req = make();
        CachedPlan c{b, h1, h2, count, entries, nparts, first_share, {}, {}};
        // contiguous input ranges: the first holds first_share of the output
        // elements (0: an equal share), the others equal shares of the rest
        const double f0 = first_share > 0.0 ? first_share : 1.0 / nparts;
        size_t first = 0;
        for (int k = 0; k < nparts; ++k) {
            size_t last = req.size();
            if (k + 1 < nparts) {
                const int64_t goal =
                    (int64_t)((double)entries * (f0 + (1.0 - f0) * k / std::max(1, nparts - 1)));
                last = std::lower_bound(req.begin() + first, req.end(), goal,
                                        [](const QuartetRequest& r, int64_t v) { return r.out_off < v; }) -
                       req.begin();
            }
            if (nparts > 1 && last == first) continue;
            auto plan = std::make_unique<PlanData>();
            plan->spread_parts = nparts;
            if (nparts == 1)
                build_plan(ctx, b, req, *plan);
            else
                build_plan(ctx, b, std::vector<QuartetRequest>(req.begin() + first, req.begin() + last), *plan);
            c.parts.push_back(std::move(plan));
            c.part_end.push_back(last < req.size() ? req[last].out_off : entries);
            first = last;
        }
        cache.push_front(std::move(c));
        size_t bytes = 0;
        int kept_plans = 0;
        for (auto it = cache.begin(); it != cache.end();) {
            for (const auto& p : it->parts) bytes += p->tasks.bytes;
            if (++kept_plans > 4 || (kept_plans > 1 && bytes > (size_t(2) << 30)))
                it = cache.erase(it);
            else
                ++it;
        }
    } else {
        cache.splice(cache.begin(), cache, hit);  // most recently used first
    }
    return cache.front();
}

template <typename Make>
PlanData& lookup_plan(gx_context* ctx, gx_basis* b, uint64_t h1, uint64_t h2, int64_t count, int64_t entries,
                      Make&& make) {
    return *lookup_parts(ctx, b, h1, h2, count, entries, 1, std::forward<Make>(make)).parts[0];
}

// Host-output calls into page-locked memory copy each class's blocks as the
// class finishes (through the mapped address).  Where the buffer has no
// usable mapped address, outputs of at least kOverlapEntries complex elements
// (1 GiB) are evaluated as kAutoCopyParts input ranges instead, the first
// holding kAutoFirstShare of the output, its copy overlapping the evaluation
// of the second.  Ranges measured on the 12-atom molecule (4.2 GB, calls of
// 77.7 ms unsplit): two equal ranges 75.9 ms, first share 0.6 / 0.7 / 0.8
// 74.2 / 73.5 / 74.1 ms, three or four ranges 75-77 ms (the split costs
// kernel time); per-class copies 67.8 ms.  gx_context_set_copy_parts chooses.
constexpr int64_t kOverlapEntries = int64_t(1) << 26;
constexpr int kAutoCopyParts = 2;
constexpr double kAutoFirstShare = 0.7;

int eri_batch_impl(gx_context* ctx, gx_basis* b, const double* B, const double* O, const uint32_t* quartets,
                   int64_t nq, int precision, double mixed_cutoff, double screening, uint32_t* kept,
                   int64_t* offsets, void* out, bool out_is_device, int64_t capacity, gx_eri_stats* stats,
                   bool cache_plan = true) {
    return guarded([&] {
        if (precision != GX_PRECISION_FP64 && precision != GX_PRECISION_MIXED && precision != GX_PRECISION_FP64_EXACT)
            raise(GX_EINVAL, "precision must be GX_PRECISION_FP64, GX_PRECISION_MIXED or GX_PRECISION_FP64_EXACT");
        if (precision == GX_PRECISION_MIXED && !(std::isfinite(mixed_cutoff) && mixed_cutoff >= 0.0))
            raise(GX_EINVAL, "mixed_cutoff must be finite and non-negative");
        if (!ctx || !b) raise(GX_EINVAL, "null context or basis");
        check_field(B, O);
        if (!std::isfinite(screening) || screening < 0.0)
            raise(GX_EINVAL, "ERI screening threshold must be finite and non-negative");
        validate_quartets(b, quartets, nq);
        std::lock_guard<std::mutex> lock(ctx->mu);
        const auto t0 = std::chrono::steady_clock::now();
        GX_CUDA(cudaSetDevice(ctx->device));
        std::vector<double> q;
        if (screening > 0.0) q = schwarz_values(ctx, b, B, O);
        auto keep = [&](const uint32_t* x) {
            return !(screening > 0.0 && q[(size_t)x[0] * b->ns + x[1]] * q[(size_t)x[2] * b->ns + x[3]] < screening);
        };
        // pass 1 (parallel over chunks): kept quartets, offsets and the
        // plan-cache key (per-chunk hashes combined in chunk order)
        std::vector<int64_t> nao(b->ns);
        for (int k = 0; k < b->ns; ++k) nao[k] = b->nao_of(k);
        constexpr int64_t kChunk = 1 << 16;
        const int64_t nchunk = (nq + kChunk - 1) / kChunk;
        std::vector<int64_t> ccount(nchunk + 1, 0), centries(nchunk + 1, 0);
        std::vector<uint64_t> ch1(nchunk), ch2(nchunk);
#pragma omp parallel for schedule(static)
        for (int64_t c = 0; c < nchunk; ++c) {
            int64_t n = 0, e = 0;
            uint64_t a = 0x243F6A8885A308D3ull, z = 0x13198A2E03707344ull;
            for (int64_t i = c * kChunk; i < std::min(nq, (c + 1) * kChunk); ++i) {
                const uint32_t* x = quartets + 4 * i;
                if (!keep(x)) continue;
                uint64_t v0, v1;
                std::memcpy(&v0, x, 8);
                std::memcpy(&v1, x + 2, 8);
                a = (((a ^ v0) * 0x9E3779B97F4A7C15ull) ^ v1) * 0xBF58476D1CE4E5B9ull;
                a ^= a >> 31;
                z = (z + v0 * 0xC2B2AE3D27D4EB4Full + (v1 ^ (uint64_t)n)) * 0x94D049BB133111EBull;
                z ^= z >> 29;
                e += nao[x[0]] * nao[x[1]] * nao[x[2]] * nao[x[3]];
                ++n;
            }
            ccount[c + 1] = n;
            centries[c + 1] = e;
            ch1[c] = a;
            ch2[c] = z;
        }
        uint64_t h1 = 0x452821E638D01377ull, h2 = 0xBE5466CF34E90C6Cull;
        for (int64_t c = 0; c < nchunk; ++c) {
            h1 = ((h1 ^ ch1[c]) * 0x9E3779B97F4A7C15ull) ^ (uint64_t)ccount[c + 1];
            h2 = (h2 + ch2[c] * 0xC2B2AE3D27D4EB4Full) ^ (h2 >> 29);
            ccount[c + 1] += ccount[c];
            centries[c + 1] += centries[c];
        }
        const int64_t count = ccount[nchunk], off = centries[nchunk];
        // pass 2 (parallel): kept quartets and packed offsets.  With a cached
        // plan it runs on the host while the device evaluates.
        bool pass2_done = false;
        auto pass2 = [&] {
            if (pass2_done) return;
#pragma omp parallel for schedule(static)
            for (int64_t c = 0; c < nchunk; ++c) {
                int64_t k = ccount[c], o = centries[c];
                for (int64_t i = c * kChunk; i < std::min(nq, (c + 1) * kChunk); ++i) {
                    const uint32_t* x = quartets + 4 * i;
                    if (!keep(x)) continue;
                    if (kept) std::memcpy(kept + 4 * k, x, 4 * sizeof(uint32_t));
                    offsets[k] = o;
                    o += nao[x[0]] * nao[x[1]] * nao[x[2]] * nao[x[3]];
                    ++k;
                }
            }
            offsets[count] = off;
            pass2_done = true;
        };
        const int64_t screened = nq - count;
        if (off > capacity) raise(GX_ELENGTH, "ERI output buffer is too small");
        double2* dout;
        if (out_is_device) {
            dout = static_cast<double2*>(out);
        } else {
            ctx->out.reserve(std::max<int64_t>(off, 1) * sizeof(double2));
            dout = ctx->out.as<double2>();
        }
        float ms = 0.f, copy_ms = 0.f;
        double prepare_ms = 0.0;
        int64_t nprim = 0, evaluated[2] = {0, 0};
        if (count) {
            // host output in page-locked memory: the copy of each output range
            // overlaps the evaluation of the next ones
            // page-locked host output: copied by the SMs through its mapped
            // address (16-byte aligned), in ranges that overlap the evaluation
            int nparts = 1;
            void* mapped = nullptr;
            if (!out_is_device && off > 0) {
                cudaPointerAttributes attr{};
                if (cudaPointerGetAttributes(&attr, out) == cudaSuccess && attr.type == cudaMemoryTypeHost) {
                    if (attr.devicePointer && !(reinterpret_cast<uintptr_t>(attr.devicePointer) & 15))
                        mapped = attr.devicePointer;
                    if (ctx->copy_parts > 1 || (ctx->copy_parts == 0 && !mapped && off >= kOverlapEntries))
                        nparts = ctx->copy_parts > 0 ? ctx->copy_parts : kAutoCopyParts;
                } else {
                    (void)cudaGetLastError();
                }
            }
            // the default with a mapped output: every class's blocks copied
            // right after the class, overlapping the other classes
            const bool class_copies = mapped && ctx->copy_parts == 0;
            CachedPlan transient;  // the plan of a call that does not cache it
            CachedPlan& cp = lookup_parts(ctx, b, h1, h2, count, off, nparts, [&] {
                pass2();
                std::vector<QuartetRequest> req((size_t)count);
#pragma omp parallel for schedule(static)
                for (int64_t c = 0; c < nchunk; ++c) {
                    int64_t k = ccount[c];
                    for (int64_t i = c * kChunk; i < std::min(nq, (c + 1) * kChunk); ++i) {
                        const uint32_t* x = quartets + 4 * i;
                        if (!keep(x)) continue;
                        req[k] = QuartetRequest{x[0], x[1], x[2], x[3], offsets[k]};
                        ++k;
                    }
                }
                return req;
            }, nparts == 1 ? 0.0 : (ctx->copy_parts == 0 ? kAutoFirstShare : ctx->copy_first),
            cache_plan ? nullptr : &transient);
            const size_t np = cp.parts.size();
            cudaStream_t s = ctx->stream;
            std::vector<unsigned long long*> counters(np, nullptr);
            for (size_t r = 0; r < np; ++r) {
                PlanData& plan = *cp.parts[r];
                apply_recorded_tuning(ctx, b, precision, plan);
                nprim += plan.primitive_quartets;
                if (stats) {
                    plan.counters.reserve(std::max<size_t>(2 * plan.classes.size(), 2) * sizeof(unsigned long long));
                    counters[r] = plan.counters.as<unsigned long long>();
                }
            }
            struct Ev {
                cudaEvent_t a = nullptr, b = nullptr, c = nullptr;
                ~Ev() {
                    if (a) cudaEventDestroy(a);
                    if (b) cudaEventDestroy(b);
                    if (c) cudaEventDestroy(c);
                }
            } ev;
            GX_CUDA(cudaEventCreate(&ev.a));
            GX_CUDA(cudaEventCreate(&ev.b));
            GX_CUDA(cudaEventCreate(&ev.c));
            prepare_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
            GX_CUDA(cudaEventRecord(ev.a, s));
            if (np == 1) {
                execute_plan(ctx, b, B, O, *cp.parts[0], dout, precision, mixed_cutoff, counters[0], false,
                             class_copies ? mapped : nullptr);
                GX_CUDA(cudaEventRecord(ev.b, s));
                if (class_copies) {
                    // (copied with the classes)
                } else if (mapped) {
                    GX_CUDA(gx::launch_host_copy(mapped, dout, off * (int64_t)sizeof(double2), kHostCopyBlocks, s));
                } else if (!out_is_device && off) {
                    GX_CUDA(cudaMemcpyAsync(out, dout, off * sizeof(double2), cudaMemcpyDeviceToHost, s));
                }
            } else {
                FieldPairs& fp = field_pairs(b, B, O);
                const gx::EriDev dev = make_dev(ctx, b, fp, dout, precision, mixed_cutoff);
                enqueue_parts_with_copies(ctx, dev, cp, precision, counters, dout, out, mapped, ev.b);
            }
            GX_CUDA(cudaEventRecord(ev.c, s));
            pass2();  // overlaps the device work
            GX_CUDA(cudaEventSynchronize(ev.c));
            GX_CUDA(cudaEventElapsedTime(&ms, ev.a, ev.b));
            GX_CUDA(cudaEventElapsedTime(&copy_ms, ev.b, ev.c));
            check_status(ctx);
            if (stats) {
                for (size_t r = 0; r < np; ++r) {
                    const PlanData& plan = *cp.parts[r];
                    std::vector<unsigned long long> c(2 * plan.classes.size());
                    if (!c.empty())
                        GX_CUDA(cudaMemcpy(c.data(), counters[r], c.size() * sizeof(unsigned long long),
                                           cudaMemcpyDeviceToHost));
                    for (size_t i = 0; i < plan.classes.size(); ++i) {
                        evaluated[0] += (int64_t)c[2 * i];
                        evaluated[1] += (int64_t)c[2 * i + 1];
                    }
                }
            }
        } else {
            pass2();
        }
        GX_CUDA(cudaStreamSynchronize(ctx->stream));
        if (stats) {
            stats->requested = nq;
            stats->computed = count;
            stats->screened = screened;
            stats->primitive_quartets = evaluated[0] + evaluated[1];
            stats->fp32_primitive_quartets = evaluated[1];
            stats->skipped_primitive_quartets = nprim - evaluated[0] - evaluated[1];
            stats->kernel_ms = ms;
            stats->prepare_ms = prepare_ms;
            stats->copy_ms = copy_ms;
            stats->call_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        }
    });
}

// ---------------------------------------------------------------------------
// packed requests: several (basis, field, quartet list) in one execution
// ---------------------------------------------------------------------------

// Primitive-pair records of several (basis, field) requests side by side:
// each request's records keep their layout at a pair base and an E~ base,
// with the record indices (order) and E~ offsets (Eoff) shifted by them, and
// the primitive counts of their segmented shells at a segment base.
struct PackedPairs {
    DeviceBuffer nprim, p, Pr, Pi, F, Eoff, Epool, bound, Epool32, order, sbound, g32;
    int npp = 0, nseg = 0;
};

void pack_pairs(gx_context* ctx, const std::vector<gx_basis*>& bases, const double* B, const double* O,
                PackedPairs& pk, std::vector<int>& seg_base, std::vector<int>& pair_base) {
    cudaStream_t st = ctx->stream;
    int64_t npp = 0, nseg = 0, E = 0;
    for (gx_basis* b : bases) {
        npp += b->npp;
        nseg += b->nseg;
        E += b->Etotal;
    }
    if (npp > (int64_t)INT32_MAX || nseg > (int64_t)INT32_MAX) raise(GX_ELENGTH, "packed requests are too large");
    const size_t n = std::max<int64_t>(npp, 1), e = std::max<int64_t>(E, 1);
    pk.p.reserve(n * sizeof(double));
    pk.Pr.reserve(3 * n * sizeof(double));
    pk.Pi.reserve(3 * n * sizeof(double));
    pk.F.reserve(n * sizeof(double2));
    pk.Eoff.reserve(n * sizeof(long long));
    pk.bound.reserve(n * sizeof(double));
    pk.order.reserve(n * sizeof(int));
    pk.sbound.reserve(n * sizeof(float));
    pk.g32.reserve(2 * n * sizeof(float4));
    pk.Epool.reserve(e * sizeof(double2));
    pk.Epool32.reserve(e * sizeof(float2));
    std::vector<int> nprim;
    seg_base.clear();
    pair_base.clear();
    int64_t pb = 0, eb = 0;
    for (size_t r = 0; r < bases.size(); ++r) {
        gx_basis* b = bases[r];
        seg_base.push_back((int)nprim.size());
        pair_base.push_back((int)pb);
        nprim.insert(nprim.end(), b->seg_nprim.begin(), b->seg_nprim.end());
        FieldPairs& fp = field_pairs(b, B + 3 * r, O + 3 * r);
        const int64_t m = b->npp;
        auto cp = [&](DeviceBuffer& dst, const DeviceBuffer& src, size_t elem, int64_t first, int64_t count) {
            if (count > 0)
                GX_CUDA(cudaMemcpyAsync(static_cast<char*>(dst.ptr) + first * elem, src.ptr, count * elem,
                                        cudaMemcpyDeviceToDevice, st));
        };
        cp(pk.p, fp.p, sizeof(double), pb, m);
        cp(pk.Pr, fp.Pr, 3 * sizeof(double), pb, m);
        cp(pk.Pi, fp.Pi, 3 * sizeof(double), pb, m);
        cp(pk.F, fp.F, sizeof(double2), pb, m);
        cp(pk.bound, fp.bound, sizeof(double), pb, m);
        cp(pk.sbound, fp.sbound, sizeof(float), pb, m);
        cp(pk.g32, fp.g32, 2 * sizeof(float4), pb, m);
        cp(pk.Epool, fp.Epool, sizeof(double2), eb, b->Etotal);
        cp(pk.Epool32, fp.Epool32, sizeof(float2), eb, b->Etotal);
        GX_CUDA(gx::launch_offset_copy(pk.order.as<int>() + pb, fp.order.as<int>(), m, (int)pb, st));
        GX_CUDA(gx::launch_offset_copy(pk.Eoff.as<long long>() + pb, b->d_Eoff.as<long long>(), m, (long long)eb,
                                       st));
        // the next request's field_pairs may rewrite this basis's records
        // (same basis, other field): the copies above come first on the stream
        pb += m;
        eb += b->Etotal;
    }
    upload(pk.nprim, nprim, st);
    pk.npp = (int)npp;
    pk.nseg = (int)nseg;
}

}  // namespace

extern "C" int gx_eri_batch_packed(gx_context* ctx, int nreq, gx_basis* const* bases, const double* B,
                                   const double* O, const uint32_t* const* quartets, const int64_t* nq, int precision,
                                   double mixed_cutoff, int64_t* const* offsets, double* const* values,
                                   const int64_t* capacity, double* kernel_ms) {
    return guarded([&] {
        if (!ctx || nreq < 0 || (nreq > 0 && (!bases || !B || !O || !quartets || !nq || !offsets || !values ||
                                               !capacity)))
            raise(GX_EINVAL, "null argument");
        if (precision != GX_PRECISION_FP64 && precision != GX_PRECISION_MIXED && precision != GX_PRECISION_FP64_EXACT)
            raise(GX_EINVAL, "precision must be GX_PRECISION_FP64, GX_PRECISION_MIXED or GX_PRECISION_FP64_EXACT");
        if (precision == GX_PRECISION_MIXED && !(std::isfinite(mixed_cutoff) && mixed_cutoff >= 0.0))
            raise(GX_EINVAL, "mixed_cutoff must be finite and non-negative");
        for (int r = 0; r < nreq; ++r) {
            if (!bases[r] || bases[r]->ctx != ctx) raise(GX_EINVAL, "every basis must belong to the context");
            check_field(B + 3 * r, O + 3 * r);
            if (nq[r] < 0 || (nq[r] > 0 && !quartets[r])) raise(GX_EINVAL, "null quartet list");
            validate_quartets(bases[r], quartets[r], nq[r]);
        }
        if (kernel_ms) *kernel_ms = 0.0;
        if (nreq == 0) return;
        std::lock_guard<std::mutex> lock(ctx->mu);
        GX_CUDA(cudaSetDevice(ctx->device));
        // blocks of every request at its own output base, offsets relative to it
        std::vector<std::vector<QuartetRequest>> reqs(nreq);
        std::vector<int64_t> base(nreq + 1, 0);
        for (int r = 0; r < nreq; ++r) {
            const gx_basis* b = bases[r];
            int64_t o = 0;
            reqs[r].reserve((size_t)nq[r]);
            for (int64_t i = 0; i < nq[r]; ++i) {
                const uint32_t* x = quartets[r] + 4 * i;
                offsets[r][i] = o;
                reqs[r].push_back({x[0], x[1], x[2], x[3], o});
                o += b->nao_of(x[0]) * b->nao_of(x[1]) * b->nao_of(x[2]) * b->nao_of(x[3]);
            }
            offsets[r][nq[r]] = o;
            if (o > capacity[r]) raise(GX_ELENGTH, "ERI output buffer is too small");
            base[r + 1] = base[r] + o;
        }
        std::vector<gx_basis*> bv(bases, bases + nreq);
        PackedPairs pk;
        std::vector<int> seg_base, pair_base;
        pack_pairs(ctx, bv, B, O, pk, seg_base, pair_base);
        std::vector<PlanPart> parts;
        for (int r = 0; r < nreq; ++r) parts.push_back({bases[r], &reqs[r], seg_base[r], pair_base[r], base[r]});
        PlanData plan;
        build_plan_parts(ctx, parts, plan);
        const int64_t total = base[nreq];
        ctx->out.reserve(std::max<int64_t>(total, 1) * sizeof(double2));
        gx::EriDev dev = make_dev(ctx, bases[0], field_pairs(bases[0], B, O), ctx->out.as<double2>(), precision,
                                  mixed_cutoff);
        dev.basis = gx::BasisDev{};
        dev.basis.ns = pk.nseg;
        dev.basis.nprim = pk.nprim.as<int>();
        dev.pairs = gx::PairData{pk.npp,
                                 pk.p.as<double>(),
                                 pk.Pr.as<double>(),
                                 pk.Pi.as<double>(),
                                 pk.F.as<double2>(),
                                 pk.Eoff.as<long long>(),
                                 pk.Epool.as<double2>(),
                                 pk.bound.as<double>(),
                                 pk.Epool32.as<float2>(),
                                 pk.order.as<int>(),
                                 pk.sbound.as<float>(),
                                 pk.g32.as<float4>()};
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        if (kernel_ms) {
            GX_CUDA(cudaEventCreate(&e0));
            GX_CUDA(cudaEventCreate(&e1));
            GX_CUDA(cudaEventRecord(e0, ctx->stream));
        }
        if (plan.ntask) enqueue_plan(ctx, dev, plan, precision, nullptr, false);
        if (kernel_ms) GX_CUDA(cudaEventRecord(e1, ctx->stream));
        for (int r = 0; r < nreq; ++r)
            if (base[r + 1] > base[r])
                GX_CUDA(cudaMemcpyAsync(values[r], ctx->out.as<double2>() + base[r],
                                        (base[r + 1] - base[r]) * sizeof(double2), cudaMemcpyDeviceToHost,
                                        ctx->stream));
        GX_CUDA(cudaStreamSynchronize(ctx->stream));
        if (kernel_ms) {
            float ms = 0.0f;
            GX_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            *kernel_ms = ms;
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
        }
        check_status(ctx);
    });
}

extern "C" int gx_context_set_copy_parts(gx_context* ctx, int parts, double first_share) {
    return guarded([&] {
        if (!ctx) raise(GX_EINVAL, "null context");
        if (parts < 0 || parts > 64) raise(GX_EINVAL, "copy parts must be in [0, 64]");
        if (!(first_share >= 0.0 && first_share < 1.0)) raise(GX_EINVAL, "first_share must be in [0, 1)");
        std::lock_guard<std::mutex> lock(ctx->mu);
        ctx->copy_parts = parts;
        ctx->copy_first = first_share;
    });
}

int gx_context_set_stable_launch(gx_context* ctx, int stable) {
    return guarded([&] {
        if (!ctx) raise(GX_EINVAL, "null context");
        std::lock_guard<std::mutex> lock(ctx->mu);
        ctx->stable_launch = stable != 0;
        drop_cached_plans(ctx, nullptr);  // cached plans were built under the other setting
        ctx->column_plans.clear();
        ctx->column_plan_bytes = 0;
    });
}

namespace {

// ---------------------------------------------------------------------------
// ERI centre derivatives
// ---------------------------------------------------------------------------

// Exponent-dependent factor of the primitive normalisation,
// g(alpha, l) = (2 alpha / pi)^{3/4} (4 alpha)^{l/2}; the component factor
// prod_x ((2 l_x - 1)!!)^{-1/2} is applied by the combine kernel.
double norm_radial(double alpha, int l) {
    return std::exp(0.75 * std::log(2.0 * alpha / M_PI) + 0.5 * l * std::log(4.0 * alpha));
}

// Derived-shell groups of the centre-derivative basis.
enum { kDerivZ = 0, kDerivU = 1, kDerivD = 2 };

// The centre-derivative basis of `b`: shells 0..ns-1 are the shells of b;
// then, for every shell s with l <= 15, Z_s (l + 1, coefficients
// w g(alpha, l) 2 alpha) and U_s (l + 1, coefficients w g(alpha, l)), and for
// l >= 1 D_s (l - 1, coefficients w g(alpha, l)), all with raw primitives
// (no Cartesian normalisation).  A raw shell of b keeps g = 1.  Built on first
// use and kept with b; deriv_index[3 ns] maps (group, s) to the derived shell.
gx_basis* derivative_basis(gx_context* ctx, gx_basis* b, std::vector<int>& index) {
    const int ns = b->ns;
    std::vector<double> centers(b->center);
    std::vector<int> l(b->l), np(b->nprim), nc(b->ncontr), raw(b->raw);
    std::vector<double> exps(b->exps), coefs(b->coefs);
    index.assign(3 * (size_t)ns, -1);
    int next = ns;
    for (int g = 0; g < 3; ++g) {
        size_t eo = 0, co = 0;
        for (int s = 0; s < ns; ++s) {
            const int ls = b->l[s];
            const bool present = g == kDerivD ? ls >= 1 : ls <= 15;
            if (present) {
                index[(size_t)g * ns + s] = next++;
                for (int k = 0; k < 3; ++k) centers.push_back(b->center[3 * s + k]);
                l.push_back(g == kDerivD ? ls - 1 : ls + 1);
                np.push_back(b->nprim[s]);
                nc.push_back(b->ncontr[s]);
                raw.push_back(1);
                for (int p = 0; p < b->nprim[s]; ++p) exps.push_back(b->exps[eo + p]);
                for (int x = 0; x < b->ncontr[s]; ++x)
                    for (int p = 0; p < b->nprim[s]; ++p) {
                        const double alpha = b->exps[eo + p];
                        double c = b->coefs[co + (size_t)x * b->nprim[s] + p];
                        if (!b->raw[s]) c *= norm_radial(alpha, ls);
                        if (g == kDerivZ) c *= 2.0 * alpha;
                        coefs.push_back(c);
                    }
            }
            eo += b->nprim[s];
            co += (size_t)b->nprim[s] * b->ncontr[s];
        }
    }
    if (!b->deriv) {
        b->deriv = new_basis(ctx, next, centers.data(), l.data(), np.data(), nc.data(), exps.data(), coefs.data(),
                             raw.data());
        std::vector<int> sl(b->l), sn(b->ncontr), sr(b->raw);
        upload(b->d_shell_l, sl, ctx->stream);
        upload(b->d_shell_ncontr, sn, ctx->stream);
        upload(b->d_shell_raw, sr, ctx->stream);
        upload(b->d_shell_center, b->center, ctx->stream);
        b->shell_inv2a.assign(ns, 0.0);
        size_t e = 0;
        for (int s2 = 0; s2 < ns; ++s2) {
            if (b->nprim[s2] == 1 && b->l[s2] <= 15) b->shell_inv2a[s2] = 1.0 / (2.0 * b->exps[e]);
            e += b->nprim[s2];
        }
        upload(b->d_shell_inv2a, b->shell_inv2a, ctx->stream);
    }
    return b->deriv.get();
}

// Index of Cartesian component k in the reference order (x descending, then y).
int comp_index_host(const std::array<int, 3>& k) {
    const int m = k[1] + k[2];
    return m * (m + 1) / 2 + k[2];
}

// Derivative-density Schwarz factors of every ordered shell pair
// (EriDerivativeSchwarzBounds, src/derivatives.cpp:1307-1372).  For
// primitives a, b of components l_a, l_b with coefficients N(alpha, l),
//   n(a', b') = N_a N_b sqrt|(b' a'|a' b')|  (unit raw primitives a', b'),
// slot s of (a, b), axis x:
//   2 alpha n(+1_x) + l_x n(-1_x) + sum_c |(B x e_x)_c| / 2 (n(+1_c) + |R_c| n),
// contracted with |w_a w_b| over primitive pairs and maximised over
// components, contractions, slots and axes; padded by (1 + 128 eps) and one ulp.
// The diagonal integrals are FP64-exact blocks of the bound basis through the
// class kernels, gathered on the device.
void derivative_schwarz_impl(gx_context* ctx, gx_basis* b, const double* B, const double* O, double* values) {
    const int ns = b->ns;
    std::vector<int> goff(ns + 1, 0);  // first global primitive of each shell
    for (int s = 0; s < ns; ++s) goff[s + 1] = goff[s] + b->nprim[s];
    std::vector<int> eoff(ns + 1, 0), coff(ns + 1, 0);
    for (int s = 0; s < ns; ++s) {
        eoff[s + 1] = eoff[s] + b->nprim[s];
        coff[s + 1] = coff[s] + b->nprim[s] * b->ncontr[s];
    }
    if (!b->bound) {
        std::vector<double> centers, exps, coefs;
        std::vector<int> l, np, nc, raw;
        b->bound_index.assign(3 * (size_t)goff[ns], -1);
        for (int s = 0; s < ns; ++s)
            for (int p = 0; p < b->nprim[s]; ++p)
                for (int v = 0; v < 3; ++v) {
                    const int lv = v == 0 ? b->l[s] : (v == 1 ? b->l[s] + 1 : b->l[s] - 1);
                    if (lv < 0 || lv > 16) continue;
                    b->bound_index[3 * (size_t)(goff[s] + p) + v] = (int)l.size();
                    for (int k = 0; k < 3; ++k) centers.push_back(b->center[3 * s + k]);
                    l.push_back(lv);
                    np.push_back(1);
                    nc.push_back(1);
                    raw.push_back(1);
                    exps.push_back(b->exps[eoff[s] + p]);
                    coefs.push_back(1.0);
                }
        b->bound = new_basis(ctx, (int)l.size(), centers.data(), l.data(), np.data(), nc.data(), exps.data(),
                             coefs.data(), raw.data());
    }
    gx_basis* bb = b->bound.get();
    // variants (left, right) of the diagonal blocks (right left | left right)
    static const int kVar[5][2] = {{0, 0}, {1, 0}, {2, 0}, {0, 1}, {0, 2}};
    // per unordered shell pair a <= c, primitive pair (p, q), variant: offset of
    // its n_right x n_left diagonal values [right comp][left comp] (-1: absent)
    std::vector<int64_t> pair_first((size_t)ns * ns, -1);
    std::vector<QuartetRequest> req;
    std::vector<long long> didx;
    std::vector<int64_t> dpos;  // per (pair, p, q, variant) in order
    int64_t off = 0;
    for (int a = 0; a < ns; ++a)
        for (int c = a; c < ns; ++c) {
            pair_first[(size_t)a * ns + c] = (int64_t)dpos.size();
            for (int p = 0; p < b->nprim[a]; ++p)
                for (int q = 0; q < b->nprim[c]; ++q)
                    for (int v = 0; v < 5; ++v) {
                        const int sl = b->bound_index[3 * (size_t)(goff[a] + p) + kVar[v][0]];
                        const int sr = b->bound_index[3 * (size_t)(goff[c] + q) + kVar[v][1]];
                        if (sl < 0 || sr < 0) {
                            dpos.push_back(-1);
                            continue;
                        }
                        const int64_t nl = gx::ncart(bb->l[sl]), nr = gx::ncart(bb->l[sr]);
                        req.push_back({(uint32_t)sr, (uint32_t)sl, (uint32_t)sl, (uint32_t)sr, off});
                        dpos.push_back((int64_t)didx.size());
                        for (int64_t cr = 0; cr < nr; ++cr)
                            for (int64_t cl = 0; cl < nl; ++cl)
                                didx.push_back(off + ((cr * nl + cl) * nl + cl) * nr + cr);
                        off += nl * nl * nr * nr;
                    }
        }
    std::vector<double> diag(didx.size());
    if (!req.empty()) {
        ctx->scratch_a.reserve(std::max<int64_t>(off, 1) * sizeof(double2));
        run_quartets(ctx, bb, B, O, req, ctx->scratch_a.as<double2>(), nullptr, nullptr, GX_PRECISION_FP64_EXACT);
        ctx->scratch_b.reserve(didx.size() * sizeof(long long));
        ctx->scratch_c.reserve(didx.size() * sizeof(double));
        GX_CUDA(cudaMemcpyAsync(ctx->scratch_b.ptr, didx.data(), didx.size() * sizeof(long long),
                                cudaMemcpyHostToDevice, ctx->stream));
        GX_CUDA(gx::launch_gather_abs(ctx->scratch_a.as<double2>(), ctx->scratch_b.as<long long>(),
                                      ctx->scratch_c.as<double>(), (long long)didx.size(), ctx->sm_count,
                                      ctx->stream));
        GX_CUDA(cudaMemcpyAsync(diag.data(), ctx->scratch_c.ptr, didx.size() * sizeof(double),
                                cudaMemcpyDeviceToHost, ctx->stream));
        GX_CUDA(cudaStreamSynchronize(ctx->stream));
    }
    const double eps = std::numeric_limits<double>::epsilon();
#pragma omp parallel for schedule(dynamic)
    for (int64_t pair = 0; pair < (int64_t)ns * ns; ++pair) {
        const int sa = (int)(pair / ns), sb = (int)(pair % ns);
        // blocks are stored for lo <= hi; slot 0 (left) is sa
        const int lo = std::min(sa, sb), hi = std::max(sa, sb);
        const bool swapped = sa > sb;
        const int la = b->l[sa], lb = b->l[sb];
        const auto ca_list = components(la), cb_list = components(lb);
        const int na = b->nprim[sa], nb = b->nprim[sb], xa_n = b->ncontr[sa], xb_n = b->ncontr[sb];
        double maximum = 0.0;
        std::vector<double> contracted(6 * (size_t)xa_n * xb_n);
        for (size_t ca = 0; ca < ca_list.size(); ++ca)
            for (size_t cb = 0; cb < cb_list.size(); ++cb) {
                std::fill(contracted.begin(), contracted.end(), 0.0);
                for (int pa = 0; pa < na; ++pa)
                    for (int pb = 0; pb < nb; ++pb) {
                        const double alpha_a = b->exps[eoff[sa] + pa], alpha_b = b->exps[eoff[sb] + pb];
                        const auto& A = ca_list[ca];
                        const auto& Bc = cb_list[cb];
                        const double Na = b->raw[sa] ? 1.0 : primitive_norm(alpha_a, A[0], A[1], A[2]);
                        const double Nb = b->raw[sb] ? 1.0 : primitive_norm(alpha_b, Bc[0], Bc[1], Bc[2]);
                        // n(shifted a component, variant va; shifted b component, variant vb)
                        auto n = [&](int va, const std::array<int, 3>& ka, int vb, const std::array<int, 3>& kb) {
                            // stored orientation: left = lo shell, right = hi shell
                            const int vl = swapped ? vb : va, vr = swapped ? va : vb;
                            const auto& kl = swapped ? kb : ka;
                            const auto& kr = swapped ? ka : kb;
                            const int pl = swapped ? pb : pa, pr = swapped ? pa : pb;
                            int v = 0;
                            for (; v < 5; ++v)
                                if (kVar[v][0] == vl && kVar[v][1] == vr) break;
                            const int nq_hi = b->nprim[hi];
                            const int64_t slot = pair_first[(size_t)lo * ns + hi] + ((int64_t)pl * nq_hi + pr) * 5 + v;
                            const int64_t base = dpos[slot];
                            const int llv = gx::ncart(kl[0] + kl[1] + kl[2]);
                            const int il = comp_index_host(kl), ir = comp_index_host(kr);
                            return Na * Nb * std::sqrt(diag[base + (int64_t)ir * llv + il]);
                        };
                        double pb6[6];
                        for (int slot = 0; slot < 2; ++slot) {
                            const auto& raw_ang = slot == 0 ? A : Bc;
                            const double alpha = slot == 0 ? alpha_a : alpha_b;
                            const double* R = &b->center[3 * (slot == 0 ? sa : sb)];
                            auto changed = [&](int dv, int axis) {
                                std::array<int, 3> k = raw_ang;
                                k[axis] += dv == 1 ? 1 : -1;
                                return slot == 0 ? n(dv, k, 0, Bc) : n(0, A, dv, k);
                            };
                            const double base_n = n(0, A, 0, Bc);
                            for (int axis = 0; axis < 3; ++axis) {
                                double bound = 2.0 * alpha * changed(1, axis);
                                if (raw_ang[axis] != 0) bound += (double)raw_ang[axis] * changed(2, axis);
                                double e[3] = {0.0, 0.0, 0.0};
                                e[axis] = 1.0;
                                const double ph[3] = {B[1] * e[2] - B[2] * e[1], B[2] * e[0] - B[0] * e[2],
                                                      B[0] * e[1] - B[1] * e[0]};
                                for (int c = 0; c < 3; ++c) {
                                    const double w = 0.5 * std::abs(ph[c]);
                                    if (w != 0.0) bound += w * (changed(1, c) + std::abs(R[c]) * base_n);
                                }
                                pb6[slot * 3 + axis] = bound;
                            }
                        }
                        for (int xa = 0; xa < xa_n; ++xa)
                            for (int xb = 0; xb < xb_n; ++xb) {
                                const double w = std::abs(b->coefs[coff[sa] + (size_t)xa * na + pa] *
                                                          b->coefs[coff[sb] + (size_t)xb * nb + pb]);
                                for (int k = 0; k < 6; ++k) contracted[((size_t)xa * xb_n + xb) * 6 + k] += w * pb6[k];
                            }
                    }
                for (double v : contracted) maximum = std::max(maximum, v);
            }
        values[pair] = std::nextafter(maximum * (1.0 + 128.0 * eps), INFINITY);
    }
}

// Validate nq quartets of b for derivative mode `mode` (0 centre, 1
// magnetic, 2 mixed field/centre) and write their output offsets
// (complex elements, nq + 1 values).
int64_t derivative_offsets(const gx_basis* b, int mode, const uint32_t* quartets, int64_t nq, int64_t* offsets) {
    if (nq < 0) raise(GX_EINVAL, "negative quartet count");
    if (nq > (int64_t)INT32_MAX) raise(GX_ELENGTH, "derivative batch size overflow");
    const uint32_t ns = (uint32_t)b->ns;
    const int lmax = mode == 2 ? 14 : 15, extra = mode == 2 ? 2 : 1;
    const int64_t ncomp = mode == 0 ? 12 : (mode == 1 ? 3 : 36);
    int64_t off = 0;
    for (int64_t i = 0; i < nq; ++i) {
        const uint32_t* x = quartets + 4 * i;
        int L = 0;
        int64_t size = 1;
        for (int k = 0; k < 4; ++k) {
            if (x[k] >= ns) raise(GX_ERANGE, "derivative shell quartet index is out of range");
            if (b->l[x[k]] > lmax)
                raise(GX_EINVAL, mode == 2 ? "ERI mixed derivatives support shells through l = 14"
                                           : "ERI centre derivatives support shells through l = 15");
            L += b->l[x[k]];
            size *= b->nao_of(x[k]);
        }
        if (L + extra > 32) raise(GX_EINVAL, "electron repulsion supports combined angular order through 32");
        offsets[i] = off;
        off += ncomp * size;
    }
    offsets[nq] = off;
    return off;
}

double inv_sqrt_double_factorial(int n) {
    double df = 1.0;  // (2n - 1)!!
    for (int k = 1; k <= n; ++k) df *= 2.0 * k - 1.0;
    return 1.0 / std::sqrt(df);
}

// Centre (mode 0) or magnetic (mode 1) derivative blocks of nq validated
// quartets into device memory dout at offsets; the caller holds ctx->mu.
void derivative_core(gx_context* ctx, gx_basis* b, int mode, const double* B, const double* O,
                     const uint32_t* quartets, int64_t nq, const int64_t* offsets, double2* dout, float* kernel_ms) {
    if (nq == 0) return;
    const uint32_t ns = (uint32_t)b->ns;
    std::vector<int> dix;
    gx_basis* db = derivative_basis(ctx, b, dix);
    const bool field = B[0] != 0.0 || B[1] != 0.0 || B[2] != 0.0;
    const bool has_u = mode == 1 || field;
    // derived blocks per quartet: for each slot [Z, D if l > 0] (centre
    // mode), [U]; then [plain]
    std::vector<uint32_t> dq;
    dq.reserve((size_t)nq * 4 * (mode == 1 ? 5 : (field ? 13 : 8)));
    std::vector<long long> doff((size_t)nq);
    int64_t dtotal = 0;
    for (int64_t i = 0; i < nq; ++i) {
        const uint32_t* x = quartets + 4 * i;
        doff[i] = dtotal;
        auto add = [&](int k, int g) {
            uint32_t y[4] = {x[0], x[1], x[2], x[3]};
            int64_t size = 1;
            if (g >= 0) y[k] = (uint32_t)dix[(size_t)g * ns + x[k]];
            for (int j = 0; j < 4; ++j) size *= db->nao_of(y[j]);
            dq.insert(dq.end(), y, y + 4);
            dtotal += size;
        };
        for (int k = 0; k < 4; ++k) {
            if (mode == 0) {
                add(k, kDerivZ);
                if (b->l[x[k]] > 0) add(k, kDerivD);
            }
            // centre mode: a single-primitive shell's U block is Z / (2 alpha)
            if (has_u && !(mode == 0 && b->shell_inv2a[x[k]] != 0.0)) add(k, kDerivU);
        }
        if (has_u) add(0, -1);
    }
    const int64_t dcount = (int64_t)dq.size() / 4;
    uint64_t h1 = 0x452821E638D01377ull ^ (uint64_t)dcount, h2 = 0xBE5466CF34E90C6Cull;
    for (int64_t i = 0; i < dcount; ++i) {
        uint64_t v0, v1;
        std::memcpy(&v0, &dq[4 * i], 8);
        std::memcpy(&v1, &dq[4 * i + 2], 8);
        h1 = (((h1 ^ v0) * 0x9E3779B97F4A7C15ull) ^ v1) * 0xBF58476D1CE4E5B9ull;
        h1 ^= h1 >> 31;
        h2 = (h2 + v0 * 0xC2B2AE3D27D4EB4Full + (v1 ^ (uint64_t)i)) * 0x94D049BB133111EBull;
        h2 ^= h2 >> 29;
    }
    PlanData& plan = lookup_plan(ctx, db, h1, h2, dcount, dtotal, [&] {
        std::vector<QuartetRequest> req;
        req.reserve((size_t)dcount);
        int64_t o = 0;
        for (int64_t i = 0; i < dcount; ++i) {
            const uint32_t* y = &dq[4 * i];
            req.push_back({y[0], y[1], y[2], y[3], o});
            o += db->nao_of(y[0]) * db->nao_of(y[1]) * db->nao_of(y[2]) * db->nao_of(y[3]);
        }
        return req;
    });
    apply_recorded_tuning(ctx, db, GX_PRECISION_FP64, plan);
    float ms = 0.f;
    ctx->deriv_vals.reserve(std::max<int64_t>(dtotal, 1) * sizeof(double2));
    run_plan(ctx, db, B, O, plan, ctx->deriv_vals.as<double2>(), kernel_ms ? &ms : nullptr, nullptr,
             GX_PRECISION_FP64, 0.0, nullptr);
    // metadata: quartets | offsets | derived offsets
    const size_t qbytes = ((size_t)nq * 16 + 15) / 16 * 16;
    const size_t obytes = (size_t)(nq + 1) * 8;
    ctx->deriv_meta.reserve(qbytes + obytes + (size_t)nq * 8);
    char* meta = ctx->deriv_meta.as<char>();
    GX_CUDA(cudaMemcpyAsync(meta, quartets, (size_t)nq * 16, cudaMemcpyHostToDevice, ctx->stream));
    GX_CUDA(cudaMemcpyAsync(meta + qbytes, offsets, obytes, cudaMemcpyHostToDevice, ctx->stream));
    GX_CUDA(cudaMemcpyAsync(meta + qbytes + obytes, doff.data(), (size_t)nq * 8, cudaMemcpyHostToDevice,
                            ctx->stream));
    gx::DerivCombineArgs a{};
    a.nq = (int)nq;
    a.mode = mode;
    a.field = field ? 1 : 0;
    a.quartets = reinterpret_cast<const uint32_t*>(meta);
    a.offsets = reinterpret_cast<const long long*>(meta + qbytes);
    a.derived_offsets = reinterpret_cast<const long long*>(meta + qbytes + obytes);
    a.shell_l = b->d_shell_l.as<int>();
    a.shell_ncontr = b->d_shell_ncontr.as<int>();
    a.shell_raw = b->d_shell_raw.as<int>();
    a.shell_center = b->d_shell_center.as<double>();
    a.shell_inv2a = b->d_shell_inv2a.as<double>();
    a.derived = ctx->deriv_vals.as<double2>();
    a.out = dout;
    for (int k = 0; k < 3; ++k) {
        a.B[k] = B[k];
        a.O[k] = O[k];
    }
    for (int n = 0; n < 18; ++n) a.inv_sqrt_df[n] = inv_sqrt_double_factorial(n);
    GX_CUDA(gx::launch_deriv_combine(a, offsets[nq], ctx->sm_count, ctx->stream));
    if (kernel_ms) *kernel_ms = ms;
}

// Mixed field/centre derivatives (4, 3, 3, na, nb, nc, nd) of nq validated
// quartets: the centre derivatives of the quartets and of the four quartets
// with one slot replaced by its U shell (the latter on the derived basis,
// whose own derived basis supplies the doubly shifted shells), their plain
// blocks, and deriv_mixed_kernel's linear combination.  Caller holds ctx->mu.
void mixed_core(gx_context* ctx, gx_basis* b, const double* B, const double* O, const uint32_t* quartets,
                int64_t nq, const int64_t* offsets, double2* dout) {
    if (nq == 0) return;
    const int ns = b->ns;
    std::vector<int> dix;
    gx_basis* db = derivative_basis(ctx, b, dix);
    std::vector<uint32_t> lists[5];
    for (int t = 0; t < 5; ++t) {
        lists[t].assign(quartets, quartets + 4 * nq);
        if (t > 0)
            for (int64_t i = 0; i < nq; ++i) {
                uint32_t& s = lists[t][4 * i + (t - 1)];
                s = (uint32_t)dix[(size_t)kDerivU * ns + s];
            }
    }
    DeviceBuffer dbuf[5];
    std::vector<long long> doff(5 * (size_t)nq), eoff(5 * (size_t)nq);
    std::vector<int64_t> o(nq + 1);
    for (int t = 0; t < 5; ++t) {
        gx_basis* bt = t == 0 ? b : db;
        const int64_t tot = derivative_offsets(bt, 0, lists[t].data(), nq, o.data());
        for (int64_t i = 0; i < nq; ++i) doff[(size_t)t * nq + i] = o[i];
        dbuf[t].reserve(std::max<int64_t>(tot, 1) * sizeof(double2));
        derivative_core(ctx, bt, 0, B, O, lists[t].data(), nq, o.data(), dbuf[t].as<double2>(), nullptr);
    }
    // plain blocks of all five lists, on the derived basis (its first ns
    // shells are the shells of b)
    std::vector<QuartetRequest> req;
    req.reserve(5 * (size_t)nq);
    int64_t etot = 0;
    for (int t = 0; t < 5; ++t)
        for (int64_t i = 0; i < nq; ++i) {
            const uint32_t* y = &lists[t][4 * i];
            eoff[(size_t)t * nq + i] = etot;
            req.push_back({y[0], y[1], y[2], y[3], etot});
            etot += db->nao_of(y[0]) * db->nao_of(y[1]) * db->nao_of(y[2]) * db->nao_of(y[3]);
        }
    DeviceBuffer ebuf, meta;
    ebuf.reserve(std::max<int64_t>(etot, 1) * sizeof(double2));
    run_quartets(ctx, db, B, O, req, ebuf.as<double2>(), nullptr);
    const size_t qbytes = ((size_t)nq * 16 + 15) / 16 * 16;
    const size_t obytes = (size_t)(nq + 1) * 8;
    const size_t tbytes = 5 * (size_t)nq * 8;
    meta.reserve(qbytes + obytes + 2 * tbytes);
    char* m = meta.as<char>();
    GX_CUDA(cudaMemcpyAsync(m, quartets, (size_t)nq * 16, cudaMemcpyHostToDevice, ctx->stream));
    GX_CUDA(cudaMemcpyAsync(m + qbytes, offsets, obytes, cudaMemcpyHostToDevice, ctx->stream));
    GX_CUDA(cudaMemcpyAsync(m + qbytes + obytes, doff.data(), tbytes, cudaMemcpyHostToDevice, ctx->stream));
    GX_CUDA(cudaMemcpyAsync(m + qbytes + obytes + tbytes, eoff.data(), tbytes, cudaMemcpyHostToDevice, ctx->stream));
    gx::DerivMixedArgs a{};
    a.nq = (int)nq;
    a.quartets = reinterpret_cast<const uint32_t*>(m);
    a.offsets = reinterpret_cast<const long long*>(m + qbytes);
    a.doff = reinterpret_cast<const long long*>(m + qbytes + obytes);
    a.eoff = reinterpret_cast<const long long*>(m + qbytes + obytes + tbytes);
    for (int t = 0; t < 5; ++t) a.D[t] = dbuf[t].as<double2>();
    a.E = ebuf.as<double2>();
    a.shell_l = b->d_shell_l.as<int>();
    a.shell_ncontr = b->d_shell_ncontr.as<int>();
    a.shell_raw = b->d_shell_raw.as<int>();
    a.shell_center = b->d_shell_center.as<double>();
    a.out = dout;
    for (int k = 0; k < 3; ++k) a.O[k] = O[k];
    for (int n = 0; n < 18; ++n) a.inv_sqrt_df[n] = inv_sqrt_double_factorial(n);
    GX_CUDA(gx::launch_deriv_mixed(a, offsets[nq], ctx->sm_count, ctx->stream));
    // the local buffers are freed on return: finish their readers first
    GX_CUDA(cudaStreamSynchronize(ctx->stream));
}

// Centre (mode 0), magnetic (mode 1) or mixed (mode 2) derivatives of nq
// shell quartets: blocks (4, 3, ...), (3, ...) or (4, 3, 3, ...) of the
// reference layout at offsets[i] (complex elements), in input order.
int eri_derivative_impl(gx_context* ctx, gx_basis* b, int mode, const double* B, const double* O,
                        const uint32_t* quartets, int64_t nq, int64_t* offsets, void* out, bool out_is_device,
                        int64_t capacity, float* kernel_ms) {
    return guarded([&] {
        if (!ctx || !b) raise(GX_EINVAL, "null context or basis");
        check_field(B, O);
        const int64_t off = derivative_offsets(b, mode, quartets, nq, offsets);
        if (off > capacity) raise(GX_ELENGTH, "derivative output buffer is too small");
        std::lock_guard<std::mutex> lock(ctx->mu);
        GX_CUDA(cudaSetDevice(ctx->device));
        if (kernel_ms) *kernel_ms = 0.f;
        if (nq == 0) return;
        double2* dout;
        if (out_is_device) {
            dout = static_cast<double2*>(out);
        } else {
            ctx->out.reserve(std::max<int64_t>(off, 1) * sizeof(double2));
            dout = ctx->out.as<double2>();
        }
        if (mode == 2)
            mixed_core(ctx, b, B, O, quartets, nq, offsets, dout);
        else
            derivative_core(ctx, b, mode, B, O, quartets, nq, offsets, dout, kernel_ms);
        if (!out_is_device)
            GX_CUDA(cudaMemcpyAsync(out, dout, off * sizeof(double2), cudaMemcpyDeviceToHost, ctx->stream));
        GX_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

}  // namespace

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------

extern "C" {

const char* gx_last_error(void) { return g_error.c_str(); }
const char* gx_version(void) { return "0.1.0"; }

double gx_primitive_normalization(double exponent, int lx, int ly, int lz) {
    return primitive_norm(exponent, lx, ly, lz);
}

int gx_shell_normalize(int l, int nprim, int ncontr, const double* exps, const double* coefs_in, int normalize,
                       double* coefs_out) {
    return guarded([&] {
        if (nprim <= 0) raise(GX_EINVAL, "a shell requires at least one primitive");
        if (ncontr <= 0) raise(GX_EINVAL, "a shell requires at least one contraction");
        if (l < 0 || l > 65535) raise(GX_EINVAL, "shell angular momentum must fit non-negative uint16");
        for (int i = 0; i < nprim; ++i)
            if (!std::isfinite(exps[i]) || exps[i] <= 0.0)
                raise(GX_EINVAL, "shell exponents must be finite and positive");
        for (int i = 0; i < nprim * ncontr; ++i)
            if (!std::isfinite(coefs_in[i])) raise(GX_EINVAL, "shell coefficients must be finite");
        for (int x = 0; x < ncontr; ++x) {
            const double* c = coefs_in + (size_t)x * nprim;
            double* o = coefs_out + (size_t)x * nprim;
            bool nonzero = false;
            for (int i = 0; i < nprim; ++i) nonzero = nonzero || c[i] != 0.0;
            if (!nonzero) raise(GX_EINVAL, "a shell contraction cannot have all-zero coefficients");
            double scale = 1.0;
            if (normalize) {
                double s = 0.0;
                for (int i = 0; i < nprim; ++i)
                    for (int j = 0; j < nprim; ++j) s += c[i] * c[j] * same_center_overlap(exps[i], exps[j], l);
                if (!std::isfinite(s) || s <= 0.0)
                    raise(GX_EINVAL, "contraction has a non-positive or non-finite norm");
                scale = 1.0 / std::sqrt(s);
            }
            for (int i = 0; i < nprim; ++i) o[i] = normalize ? c[i] * scale : c[i];
        }
    });
}

}  // extern "C"

namespace {

std::mutex g_tables_mu;
std::map<int, std::weak_ptr<SharedTables>> g_tables;

// The shared tables of `device` (current), built on stream `st` by the first
// caller and completed before they are published.
std::shared_ptr<SharedTables> device_tables(int device, cudaStream_t st) {
    std::lock_guard<std::mutex> lock(g_tables_mu);
    if (auto live = g_tables[device].lock()) return live;
    auto tb = std::make_shared<SharedTables>();
    gx::GLRules gl;
    gauss_legendre(16, gl.x16, gl.w16);
    gauss_legendre(32, gl.x32, gl.w32);
    tb->gl.reserve(sizeof gl);
    GX_CUDA(cudaMemcpy(tb->gl.ptr, &gl, sizeof gl, cudaMemcpyHostToDevice));
    std::vector<uint32_t> herm(gx::herm_count(32));
    for (int s = 0; s <= 32; ++s)
        for (int k = s; k >= 0; --k)
            for (int l = s - k; l >= 0; --l) {
                const int m = s - k - l;
                herm[gx::herm_index(k, l, m)] = (uint32_t)(k | (l << 8) | (m << 16));
            }
    upload(tb->herm, herm, st);
    {
        std::vector<int2> plan;
        std::vector<int> off{0, 0};  // L = 0 has no steps
        for (int L = 1; L <= gx::REC_PLAN_MAX; ++L) {
            for (int n = L - 1; n >= 0; --n) {
                for (int dg = L - n; dg >= 1; --dg)
                    for (int k = dg; k >= 0; --k)
                        for (int l = dg - k; l >= 0; --l) {
                            const int m = dg - k - l;
                            int axis, pw, i1, i2;
                            if (k > 0) {
                                axis = 0, pw = k, i1 = gx::herm_index(k - 1, l, m);
                                i2 = k > 1 ? gx::herm_index(k - 2, l, m) : 0;
                            } else if (l > 0) {
                                axis = 1, pw = l, i1 = gx::herm_index(0, l - 1, m);
                                i2 = l > 1 ? gx::herm_index(0, l - 2, m) : 0;
                            } else {
                                axis = 2, pw = m, i1 = gx::herm_index(0, 0, m - 1);
                                i2 = m > 1 ? gx::herm_index(0, 0, m - 2) : 0;
                            }
                            plan.push_back(make_int2(gx::herm_index(k, l, m) | (i1 << 16),
                                                     i2 | (axis << 14) | ((pw - 1) << 16)));
                        }
                plan.push_back(make_int2(0, (1 << 22) | (n << 23)));
            }
            off.push_back((int)plan.size());
        }
        upload(tb->rec_plan, plan, st);
        upload(tb->rec_plan_off, off, st);
    }
    const size_t npts = (size_t)gx::BOYS_NX * gx::BOYS_NY;
    tb->boys_S.reserve(npts * gx::BOYS_TABLE_ORDERS * sizeof(double2));
    tb->boys_E0.reserve(npts * sizeof(double2));
    DeviceBuffer fails;  // [0]: points worse than 1e-13, [1]: worst relative agreement (double bits)
    fails.reserve(2 * sizeof(unsigned long long));
    GX_CUDA(cudaMemsetAsync(fails.ptr, 0, 2 * sizeof(unsigned long long), st));
    GX_CUDA(gx::launch_boys_table(tb->boys_S.as<double2>(), tb->boys_E0.as<double2>(),
                                  tb->gl.as<gx::GLRules>(), fails.as<int>(), st));
    unsigned long long words[2] = {0, 0};
    GX_CUDA(cudaMemcpyAsync(words, fails.ptr, sizeof words, cudaMemcpyDeviceToHost, st));
    GX_CUDA(cudaStreamSynchronize(st));
    double worst;
    std::memcpy(&worst, &words[1], sizeof worst);
    tb->boys_table_agreement = worst;
    g_tables[device] = tb;
    return tb;
}

}  // namespace

extern "C" {

int gx_context_create(int device, gx_context** out) {
    return guarded([&] {
        auto ctx = std::make_unique<gx_context>();
        ctx->device = device;
        GX_CUDA(cudaSetDevice(device));
        GX_CUDA(cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device));
        GX_CUDA(cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking));
        ctx->stream = ctx->own_stream;
        ctx->status.reserve(sizeof(gx::DevStatus));
        ctx->t = device_tables(device, ctx->stream);
        *out = ctx.release();
    });
}

void gx_context_destroy(gx_context* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    drop_cached_plans(ctx, nullptr);
    ctx->pair_classes.clear();
    for (auto st : ctx->aux) cudaStreamDestroy(st);
    for (auto ev : ctx->aux_done) cudaEventDestroy(ev);
    if (ctx->fork) cudaEventDestroy(ctx->fork);
    if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
    if (ctx->copy_done) cudaEventDestroy(ctx->copy_done);
    for (auto st : ctx->class_copy) cudaStreamDestroy(st);
    for (auto ev : ctx->class_copy_done) cudaEventDestroy(ev);
    if (ctx->class_done) cudaEventDestroy(ctx->class_done);
    cudaStreamDestroy(ctx->own_stream);
    delete ctx;
}

int gx_basis_create(gx_context* ctx, int nshell, const double* centers, const int* l, const int* nprim,
                    const int* ncontr, const double* exponents, const double* coefs, const int* raw, gx_basis** out) {
    return guarded([&] {
        if (!ctx) raise(GX_EINVAL, "null context");
        if (nshell < 0) raise(GX_EINVAL, "negative shell count");
        std::lock_guard<std::mutex> lock(ctx->mu);
        GX_CUDA(cudaSetDevice(ctx->device));
        *out = new_basis(ctx, nshell, centers, l, nprim, ncontr, exponents, coefs, raw).release();
    });
}

void gx_basis_destroy(gx_basis* b) {
    if (!b) return;
    std::lock_guard<std::mutex> lock(b->ctx->mu);
    cudaSetDevice(b->ctx->device);
    cudaStreamSynchronize(b->ctx->stream);
    // plans and tunings of the basis and of the derived bases it owns
    // (derivative bases nest: the mixed derivatives use two levels)
    std::vector<const gx_basis*> owned{b};
    for (size_t i = 0; i < owned.size(); ++i) {
        if (owned[i]->deriv) owned.push_back(owned[i]->deriv.get());
        if (owned[i]->bound) owned.push_back(owned[i]->bound.get());
    }
    for (const gx_basis* o : owned) drop_cached_plans(b->ctx, o);
    // (its Cholesky column plans go too; the byte count is a soft cap and is
    // only reset when no plan is left)
    for (auto it = b->ctx->column_plans.begin(); it != b->ctx->column_plans.end();)
        it = std::get<0>(it->first) == b ? b->ctx->column_plans.erase(it) : std::next(it);
    if (b->ctx->column_plans.empty()) b->ctx->column_plan_bytes = 0;
    delete b;
}

int64_t gx_basis_ao_count(const gx_basis* b) { return b ? b->nao : 0; }

int gx_boys(gx_context* ctx, const double* z, int64_t count, int nmax, int scaled, double* out, int* region) {
    return guarded([&] {
        if (!ctx) raise(GX_EINVAL, "null context");
        if (nmax < 0) raise(GX_EINVAL, "Boys output must contain at least F_0");
        if (nmax > 32) raise(GX_EINVAL, "complex Boys supports orders through 32");
        for (int64_t i = 0; i < 2 * count; ++i)
            if (!std::isfinite(z[i])) raise(GX_EINVAL, "complex Boys argument must be finite");
        if (count <= 0) return;
        std::lock_guard<std::mutex> lock(ctx->mu);
        GX_CUDA(cudaSetDevice(ctx->device));
        const size_t nz = (size_t)count * sizeof(double2);
        const size_t no = (size_t)count * (nmax + 1) * sizeof(double2);
        ctx->scratch_a.reserve(nz);
        ctx->scratch_b.reserve(no);
        ctx->scratch_c.reserve((size_t)count * sizeof(int));
        GX_CUDA(cudaMemcpyAsync(ctx->scratch_a.ptr, z, nz, cudaMemcpyHostToDevice, ctx->stream));
        ctx->reset_status();
        GX_CUDA(gx::launch_boys_values(ctx->scratch_a.as<double2>(), count, nmax, scaled, ctx->boys(),
                                       ctx->t->gl.as<gx::GLRules>(), ctx->scratch_b.as<double2>(),
                                       region ? ctx->scratch_c.as<int>() : nullptr,
                                       ctx->status.as<gx::DevStatus>(), ctx->stream));
        check_status(ctx);
        GX_CUDA(cudaMemcpyAsync(out, ctx->scratch_b.ptr, no, cudaMemcpyDeviceToHost, ctx->stream));
        if (region)
            GX_CUDA(cudaMemcpyAsync(region, ctx->scratch_c.ptr, count * sizeof(int), cudaMemcpyDeviceToHost,
                                    ctx->stream));
        GX_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

int gx_eri_batch(gx_context* ctx, gx_basis* basis, const double* B, const double* O, const uint32_t* quartets,
                 int64_t nq, int precision, double mixed_cutoff, double screening_threshold, uint32_t* kept,
                 int64_t* offsets, double* out, int64_t out_capacity, gx_eri_stats* stats) {
    return eri_batch_impl(ctx, basis, B, O, quartets, nq, precision, mixed_cutoff, screening_threshold, kept, offsets,
                          out, false, out_capacity, stats);
}

int gx_eri_batch_device(gx_context* ctx, gx_basis* basis, const double* B, const double* O,
                        const uint32_t* quartets, int64_t nq, int precision, double mixed_cutoff,
                        double screening_threshold, uint32_t* kept, int64_t* offsets, void* out_device,
                        int64_t out_capacity, gx_eri_stats* stats) {
    return eri_batch_impl(ctx, basis, B, O, quartets, nq, precision, mixed_cutoff, screening_threshold, kept, offsets,
                          out_device, true, out_capacity, stats);
}

int gx_eri_for_each(gx_context* ctx, gx_basis* b, const double* B, const double* O, const uint32_t* quartets,
                    int64_t nq, int precision, double mixed_cutoff, double screening, gx_quartet_consumer consumer,
                    void* user_data, gx_eri_stats* stats) {
    return guarded([&] {
        if (!consumer) raise(GX_EINVAL, "ERI quartet consumer must not be null");
        if (!ctx || !b) raise(GX_EINVAL, "null context or basis");
        if (nq < 0) raise(GX_EINVAL, "negative quartet count");
        check_field(B, O);
        if (!std::isfinite(screening) || screening < 0.0)
            raise(GX_EINVAL, "ERI screening threshold must be finite and non-negative");
        validate_quartets(b, quartets, nq);
        std::lock_guard<std::mutex> stream_lock(ctx->stream_mu);
        const auto t0 = std::chrono::steady_clock::now();
        // screening once for the whole call (src/eri.cpp:674-685)
        std::vector<uint32_t> active;
        const uint32_t* q = quartets;
        int64_t n = nq;
        if (screening > 0.0) {
            std::vector<double> bound;
            {
                std::lock_guard<std::mutex> lock(ctx->mu);
                GX_CUDA(cudaSetDevice(ctx->device));
                bound = schwarz_values(ctx, b, B, O);
            }
            const size_t ns = (size_t)b->ns;
            active.reserve((size_t)4 * nq);
            for (int64_t i = 0; i < nq; ++i) {
                const uint32_t* x = quartets + 4 * i;
                if (bound[x[0] * ns + x[1]] * bound[x[2] * ns + x[3]] < screening) continue;
                active.insert(active.end(), x, x + 4);
            }
            q = active.data();
            n = (int64_t)(active.size() / 4);
        }
        // chunks of at most kStreamChunk complex elements (a larger block alone)
        constexpr int64_t kStreamChunk = int64_t(1) << 23;
        auto elems = [&](int64_t i) {
            const uint32_t* x = q + 4 * i;
            return b->nao_of(x[0]) * b->nao_of(x[1]) * b->nao_of(x[2]) * b->nao_of(x[3]);
        };
        std::vector<int64_t> first{0};
        int64_t acc = 0, widest = 0;
        for (int64_t i = 0; i < n; ++i) {
            const int64_t e = elems(i);
            if (acc && acc + e > kStreamChunk) {
                first.push_back(i);
                widest = std::max(widest, acc);
                acc = 0;
            }
            acc += e;
        }
        widest = std::max(widest, acc);
        if (n) first.push_back(n);
        const int64_t nchunk = (int64_t)first.size() - 1;
        for (int k = 0; k < std::min<int64_t>(nchunk, 2); ++k)
            ctx->stream_host[k].reserve((size_t)std::max<int64_t>(widest, 1) * sizeof(double2));
        struct Chunk {
            std::vector<int64_t> offsets;
            gx_eri_stats st{};
            int rc = 0;
            std::string msg;
        };
        auto run = [&](int64_t k, Chunk& c) {
            const int slot = (int)(k & 1);
            const int64_t cnt = first[k + 1] - first[k];
            c.offsets.assign((size_t)cnt + 1, 0);
            c.st = gx_eri_stats{};
            // (the chunks of a long list do not displace the cached plans of other calls)
            c.rc = eri_batch_impl(ctx, b, B, O, q + 4 * first[k], cnt, precision, mixed_cutoff, 0.0, nullptr,
                                  c.offsets.data(), ctx->stream_host[slot].p, false,
                                  (int64_t)(ctx->stream_host[slot].n / sizeof(double2)), &c.st, nchunk <= 2);
            if (c.rc) c.msg = g_error;
        };
        gx_eri_stats total{};
        total.requested = nq;
        total.screened = nq - n;
        total.computed = n;
        Chunk cur, next;
        if (nchunk) run(0, cur);
        for (int64_t k = 0; k < nchunk; ++k) {
            if (cur.rc) raise(cur.rc, cur.msg);
            total.primitive_quartets += cur.st.primitive_quartets;
            total.fp32_primitive_quartets += cur.st.fp32_primitive_quartets;
            total.skipped_primitive_quartets += cur.st.skipped_primitive_quartets;
            total.kernel_ms += cur.st.kernel_ms;
            total.prepare_ms += cur.st.prepare_ms;
            total.copy_ms += cur.st.copy_ms;
            std::future<void> ahead;
            if (k + 1 < nchunk) ahead = std::async(std::launch::async, [&, k] { run(k + 1, next); });
            const double* base = static_cast<const double*>(ctx->stream_host[k & 1].p);
            int crc = 0;
            for (int64_t i = first[k]; i < first[k + 1] && !crc; ++i) {
                const uint32_t* x = q + 4 * i;
                gx_quartet_block blk;
                for (int j = 0; j < 4; ++j) {
                    blk.shells[j] = x[j];
                    blk.shape[j] = b->nao_of(x[j]);
                }
                const int64_t o = cur.offsets[(size_t)(i - first[k])];
                blk.values = base + 2 * o;
                blk.count = cur.offsets[(size_t)(i - first[k]) + 1] - o;
                crc = consumer(&blk, user_data);
            }
            if (ahead.valid()) ahead.wait();
            if (crc) raise(GX_ECONSUMER, "ERI quartet consumer returned " + std::to_string(crc));
            std::swap(cur, next);
        }
        total.call_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        if (stats) *stats = total;
    });
}

int gx_eri_center_derivatives(gx_context* ctx, gx_basis* basis, const double* B, const double* O,
                              const uint32_t* quartets, int64_t nq, int64_t* offsets, double* out,
                              int64_t out_capacity, float* kernel_ms) {
    return eri_derivative_impl(ctx, basis, 0, B, O, quartets, nq, offsets, out, false, out_capacity, kernel_ms);
}

int gx_eri_magnetic_derivatives(gx_context* ctx, gx_basis* basis, const double* B, const double* O,
                                const uint32_t* quartets, int64_t nq, int64_t* offsets, double* out,
                                int64_t out_capacity, float* kernel_ms) {
    return eri_derivative_impl(ctx, basis, 1, B, O, quartets, nq, offsets, out, false, out_capacity, kernel_ms);
}

int gx_eri_derivative_contraction(gx_context* ctx, gx_basis* basis, const double* B, const double* O,
                                  const uint32_t* quartets, int64_t nq, const int64_t* shell_atoms, int natom,
                                  int npc, const double* coulomb, int npx, const double* exchange,
                                  const double* gamma, int gamma_complex, int64_t batch_elements, double* out) {
    return guarded([&] {
        if (!ctx || !basis || !out) raise(GX_EINVAL, "null context, basis or output");
        check_field(B, O);
        gx_basis* b = basis;
        const int ns = b->ns;
        if (natom < 0) raise(GX_EINVAL, "natom must be non-negative");
        for (int s2 = 0; s2 < ns; ++s2)
            if (shell_atoms[s2] < 0 || shell_atoms[s2] >= natom) raise(GX_ERANGE, "shell atom index is out of range");
        if (npc < 0 || npx < 0) raise(GX_EINVAL, "negative density pair count");
        if (npc == 0 && npx == 0 && !gamma) raise(GX_EINVAL, "at least one density pair or gamma is required");
        if (batch_elements <= 0) raise(GX_EINVAL, "batch size must be positive");
        // canonical quartets only (src/assembly.cpp:112-114)
        for (int64_t i = 0; i < nq; ++i) {
            const uint32_t* x = quartets + 4 * i;
            for (int k = 0; k < 4; ++k)
                if (x[k] >= (uint32_t)ns) raise(GX_ERANGE, "quartet index out of range");
            const std::array<uint32_t, 4> img[4] = {{x[0], x[1], x[2], x[3]}, {x[2], x[3], x[0], x[1]},
                                                    {x[1], x[0], x[3], x[2]}, {x[3], x[2], x[1], x[0]}};
            if (*std::min_element(img, img + 4) != img[0])
                raise(GX_EINVAL, "contraction requires canonical quartets");
        }
        std::vector<int64_t> all(nq + 1);
        derivative_offsets(b, 0, quartets, nq, all.data());
        std::lock_guard<std::mutex> lock(ctx->mu);
        GX_CUDA(cudaSetDevice(ctx->device));
        if (nq == 0) return;
        const int64_t n = b->nao;
        DeviceBuffer dj, dk, dg, dstart, dbuf, meta, dpart;
        auto up = [&](DeviceBuffer& d, const void* src, size_t bytes) {
            d.reserve(std::max<size_t>(bytes, 16));
            if (bytes) GX_CUDA(cudaMemcpyAsync(d.ptr, src, bytes, cudaMemcpyHostToDevice, ctx->stream));
        };
        up(dj, coulomb, (size_t)2 * npc * n * n * sizeof(double2));
        up(dk, exchange, (size_t)2 * npx * n * n * sizeof(double2));
        if (gamma) up(dg, gamma, (size_t)n * n * n * n * (gamma_complex ? sizeof(double2) : sizeof(double)));
        up(dstart, b->ao_off.data(), (size_t)ns * sizeof(int64_t));
        std::vector<int64_t> loff;
        std::vector<double2> part;
        std::vector<std::complex<double>> acc((size_t)natom * 3, 0.0);
        for (int64_t i0 = 0; i0 < nq;) {
            int64_t i1 = i0 + 1;
            while (i1 < nq && all[i1 + 1] - all[i0] <= batch_elements) ++i1;
            const int64_t cnt = i1 - i0;
            loff.assign(cnt + 1, 0);
            const int64_t tot = derivative_offsets(b, 0, quartets + 4 * i0, cnt, loff.data());
            dbuf.reserve(std::max<int64_t>(tot, 1) * sizeof(double2));
            derivative_core(ctx, b, 0, B, O, quartets + 4 * i0, cnt, loff.data(), dbuf.as<double2>(), nullptr);
            const size_t qbytes = ((size_t)cnt * 16 + 15) / 16 * 16;
            meta.reserve(qbytes + (size_t)cnt * 8);
            GX_CUDA(cudaMemcpyAsync(meta.ptr, quartets + 4 * i0, (size_t)cnt * 16, cudaMemcpyHostToDevice,
                                    ctx->stream));
            GX_CUDA(cudaMemcpyAsync(meta.as<char>() + qbytes, loff.data(), (size_t)cnt * 8, cudaMemcpyHostToDevice,
                                    ctx->stream));
            dpart.reserve((size_t)cnt * 12 * sizeof(double2));
            gx::DerivContractArgs a{};
            a.nq = (int)cnt;
            a.quartets = meta.as<uint32_t>();
            a.offsets = reinterpret_cast<const long long*>(meta.as<char>() + qbytes);
            a.D = dbuf.as<double2>();
            a.shell_l = b->d_shell_l.as<int>();
            a.shell_ncontr = b->d_shell_ncontr.as<int>();
            a.ao_start = dstart.as<long long>();
            a.n = n;
            a.npc = npc;
            a.npx = npx;
            a.coulomb = dj.as<double2>();
            a.exchange = dk.as<double2>();
            a.gamma = gamma && gamma_complex ? dg.as<double2>() : nullptr;
            a.gamma_real = gamma && !gamma_complex ? dg.as<double>() : nullptr;
            a.partials = dpart.as<double2>();
            GX_CUDA(gx::launch_deriv_contract(a, ctx->sm_count, ctx->stream));
            part.resize((size_t)cnt * 12);
            GX_CUDA(cudaMemcpyAsync(part.data(), dpart.ptr, part.size() * sizeof(double2), cudaMemcpyDeviceToHost,
                                    ctx->stream));
            GX_CUDA(cudaStreamSynchronize(ctx->stream));
            // fixed canonical-quartet and slot order (src/assembly.cpp:151-157)
            for (int64_t r = 0; r < cnt; ++r)
                for (int slot = 0; slot < 4; ++slot) {
                    const int64_t atom = shell_atoms[quartets[4 * (i0 + r) + slot]];
                    for (int axis = 0; axis < 3; ++axis) {
                        const double2 v = part[(size_t)r * 12 + slot * 3 + axis];
                        acc[(size_t)atom * 3 + axis] += std::complex<double>(v.x, v.y);
                    }
                }
            i0 = i1;
        }
        for (size_t i = 0; i < acc.size(); ++i) {
            out[2 * i] += acc[i].real();
            out[2 * i + 1] += acc[i].imag();
        }
    });
}

int gx_eri_mixed_derivatives(gx_context* ctx, gx_basis* basis, const double* B, const double* O,
                             const uint32_t* quartets, int64_t nq, int64_t* offsets, double* out, int64_t out_capacity) {
    return eri_derivative_impl(ctx, basis, 2, B, O, quartets, nq, offsets, out, false, out_capacity, nullptr);
}

int gx_eri_derivative_schwarz(gx_context* ctx, gx_basis* basis, const double* B, const double* O, double* values,
                              double* ordinary) {
    return guarded([&] {
        if (!ctx || !basis) raise(GX_EINVAL, "null context or basis");
        check_field(B, O);
        for (int s = 0; s < basis->ns; ++s)
            if (basis->l[s] > 15) raise(GX_EINVAL, "ERI centre derivatives support shells through l = 15");
        std::lock_guard<std::mutex> lock(ctx->mu);
        GX_CUDA(cudaSetDevice(ctx->device));
        if (basis->ns == 0) return;
        derivative_schwarz_impl(ctx, basis, B, O, values);
        if (ordinary) {
            const std::vector<double> q = schwarz_values(ctx, basis, B, O);
            std::copy(q.begin(), q.end(), ordinary);
        }
    });
}

int gx_eri_center_derivatives_device(gx_context* ctx, gx_basis* basis, const double* B, const double* O,
                                     const uint32_t* quartets, int64_t nq, int64_t* offsets, void* out_device,
                                     int64_t out_capacity, float* kernel_ms) {
    return eri_derivative_impl(ctx, basis, 0, B, O, quartets, nq, offsets, out_device, true, out_capacity,
                               kernel_ms);
}

int gx_eri_shell(gx_context* ctx, gx_basis* basis, int a, int b, int c, int d, const double* B, const double* O,
                 double* out) {
    const uint32_t q[4] = {(uint32_t)a, (uint32_t)b, (uint32_t)c, (uint32_t)d};
    int64_t offsets[2];
    if (a < 0 || b < 0 || c < 0 || d < 0) return fail(GX_ERANGE, "ERI shell-quartet index is out of range");
    int64_t cap = INT64_MAX;
    return eri_batch_impl(ctx, basis, B, O, q, 1, GX_PRECISION_FP64, 0.0, 0.0, nullptr, offsets, out, false, cap,
                          nullptr);
}

int gx_schwarz(gx_context* ctx, gx_basis* b, const double* B, const double* O, double* out) {
    return guarded([&] {
        if (!ctx || !b) raise(GX_EINVAL, "null context or basis");
        check_field(B, O);
        std::lock_guard<std::mutex> lock(ctx->mu);
        GX_CUDA(cudaSetDevice(ctx->device));
        const auto q = schwarz_values(ctx, b, B, O);
        std::copy(q.begin(), q.end(), out);
    });
}

int gx_eri_full(gx_context* ctx, gx_basis* b, const double* B, const double* O, int precision, double mixed_cutoff,
                double screening, double* out) {
    return guarded([&] {
        if (precision != GX_PRECISION_FP64 && precision != GX_PRECISION_MIXED && precision != GX_PRECISION_FP64_EXACT)
            raise(GX_EINVAL, "precision must be GX_PRECISION_FP64, GX_PRECISION_MIXED or GX_PRECISION_FP64_EXACT");
        if (!ctx || !b) raise(GX_EINVAL, "null context or basis");
        check_field(B, O);
        if (!std::isfinite(screening) || screening < 0.0)
            raise(GX_EINVAL, "ERI screening threshold must be finite and non-negative");
        std::lock_guard<std::mutex> lock(ctx->mu);
        GX_CUDA(cudaSetDevice(ctx->device));
        const int64_t n = b->nao;
        std::vector<double> q;
        if (screening > 0.0) q = schwarz_values(ctx, b, B, O);
        std::vector<QuartetRequest> req;
        std::vector<long long> boff;
        std::vector<int> info;
        int64_t off = 0;
        const int ns = b->ns;
        for (int a = 0; a < ns; ++a)
            for (int bb = 0; bb < ns; ++bb)
                for (int c = 0; c < ns; ++c)
                    for (int d = 0; d < ns; ++d) {
                        const std::array<int, 4> me{a, bb, c, d};
                        const std::array<std::array<int, 4>, 3> other{
                            {{c, d, a, bb}, {bb, a, d, c}, {d, c, bb, a}}};
                        bool canonical = true;
                        for (const auto& o : other)
                            if (o < me) canonical = false;
                        if (!canonical) continue;
                        if (screening > 0.0 && q[(size_t)a * ns + bb] * q[(size_t)c * ns + d] < screening) continue;
                        req.push_back({(uint32_t)a, (uint32_t)bb, (uint32_t)c, (uint32_t)d, off});
                        boff.push_back(off);
                        const int na = (int)b->nao_of(a), nb = (int)b->nao_of(bb), nc = (int)b->nao_of(c),
                                  nd = (int)b->nao_of(d);
                        info.insert(info.end(), {(int)b->ao_off[a], (int)b->ao_off[bb], (int)b->ao_off[c],
                                                 (int)b->ao_off[d], na | (nb << 8) | (nc << 16) | (nd << 24)});
                        off += (int64_t)na * nb * nc * nd;
                    }
        ctx->out.reserve(std::max<int64_t>(off, 1) * sizeof(double2));
        const size_t full_bytes = (size_t)n * n * n * n * sizeof(double2);
        ctx->scratch_b.reserve(std::max<size_t>(full_bytes, 16));
        if (!req.empty())
            run_quartets(ctx, b, B, O, req, ctx->out.as<double2>(), nullptr, nullptr, precision, mixed_cutoff);
        GX_CUDA(cudaMemsetAsync(ctx->scratch_b.ptr, 0, full_bytes, ctx->stream));
        DeviceBuffer d_boff, d_info;
        upload(d_boff, boff, ctx->stream);
        upload(d_info, info, ctx->stream);
        GX_CUDA(gx::launch_scatter_full(ctx->out.as<double2>(), d_boff.as<long long>(), d_info.as<int>(),
                                        (int)req.size(), n, ctx->scratch_b.as<double2>(), ctx->stream));
        if (full_bytes)
            GX_CUDA(cudaMemcpyAsync(out, ctx->scratch_b.ptr, full_bytes, cudaMemcpyDeviceToHost, ctx->stream));
        GX_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

int gx_primitive_eri(gx_context* ctx, const double* exps, const double* centers, const int* angular,
                     const double* coefs, const int* normalized, const double* B, const double* O, double* out) {
    return guarded([&] {
        if (!ctx) raise(GX_EINVAL, "null context");
        check_field(B, O);
        int ls[4], L = 0;
        for (int i = 0; i < 4; ++i) {
            if (!std::isfinite(exps[i]) || exps[i] <= 0.0)
                raise(GX_EINVAL, "Gaussian exponent must be finite and positive");
            if (!std::isfinite(coefs[i])) raise(GX_EINVAL, "primitive coefficient must be finite");
            ls[i] = angular[3 * i] + angular[3 * i + 1] + angular[3 * i + 2];
            L += ls[i];
        }
        if (L > 32) raise(GX_EINVAL, "electron repulsion supports combined angular order through 32");
        // four raw (unnormalised) single-primitive shells; pick the component
        const int np[4] = {1, 1, 1, 1}, nc[4] = {1, 1, 1, 1}, raw[4] = {1, 1, 1, 1};
        const double one[4] = {1.0, 1.0, 1.0, 1.0};
        gx_basis* b = nullptr;
        int rc = gx_basis_create(ctx, 4, centers, ls, np, nc, exps, one, raw, &b);
        if (rc) raise(rc, g_error);
        std::unique_ptr<gx_basis, void (*)(gx_basis*)> guard(b, gx_basis_destroy);
        int64_t n[4], idx[4];
        for (int i = 0; i < 4; ++i) {
            n[i] = gx::ncart(ls[i]);
            const auto comps = components(ls[i]);
            idx[i] = -1;
            for (size_t k = 0; k < comps.size(); ++k)
                if (comps[k][0] == angular[3 * i] && comps[k][1] == angular[3 * i + 1] &&
                    comps[k][2] == angular[3 * i + 2])
                    idx[i] = (int64_t)k;
        }
        std::vector<double> blk(2 * n[0] * n[1] * n[2] * n[3]);
        rc = gx_eri_shell(ctx, b, 0, 1, 2, 3, B, O, blk.data());
        if (rc) raise(rc, g_error);
        const int64_t e = ((idx[0] * n[1] + idx[1]) * n[2] + idx[2]) * n[3] + idx[3];
        double scale = 1.0;
        for (int i = 0; i < 4; ++i) {
            scale *= coefs[i];
            if (normalized[i]) scale *= primitive_norm(exps[i], angular[3 * i], angular[3 * i + 1], angular[3 * i + 2]);
        }
        out[0] = blk[2 * e] * scale;
        out[1] = blk[2 * e + 1] * scale;
    });
}

int gx_nuclear_attraction(gx_context* ctx, gx_basis* b, const double* B, const double* O, int nnuc,
                          const double* charges, const double* centers, double* out) {
    return guarded([&] {
        if (!ctx || !b) raise(GX_EINVAL, "null context or basis");
        check_field(B, O);
        if (nnuc < 0) raise(GX_EINVAL, "nucleus count must be non-negative");
        for (int c = 0; c < nnuc; ++c) {
            if (!std::isfinite(charges[c]) || charges[c] <= 0.0)
                raise(GX_EINVAL, "nuclear charge must be finite and positive");
            for (int x = 0; x < 3; ++x)
                if (!std::isfinite(centers[3 * c + x])) raise(GX_EINVAL, "nuclear center values must be finite");
        }
        int lmax = 0;
        for (int s = 0; s < b->ns; ++s) lmax = std::max(lmax, b->l[s]);
        if (2 * lmax > 32) raise(GX_EINVAL, "nuclear attraction supports combined angular order through 32");
        const int nab_max = gx::ncart(lmax) * gx::ncart(lmax);
        const size_t smem = (size_t)(2 * gx::herm_count(2 * lmax) + 2 * lmax + 4 + nab_max) * sizeof(double2);
        if (smem > 200 * 1024)
            raise(GX_EINVAL, "nuclear attraction on the GPU supports shells through angular momentum 11");
        const int64_t n = b->nao;
        std::lock_guard<std::mutex> lock(ctx->mu);
        GX_CUDA(cudaSetDevice(ctx->device));
        cudaStream_t st = ctx->stream;
        if (n == 0) return;
        FieldPairs& fp = field_pairs(b, B, O);
        std::vector<long long> seg_ao(std::max(b->nseg, 1));
        for (int s = 0; s < b->ns; ++s)
            for (int x = 0; x < b->ncontr[s]; ++x)
                seg_ao[b->seg_first[s] + x] = b->ao_off[s] + (long long)x * b->ncart_of(s);
        std::vector<double> nuc(std::max(4 * nnuc, 1));
        for (int c = 0; c < nnuc; ++c) {
            nuc[c] = charges[c];
            for (int x = 0; x < 3; ++x) nuc[nnuc + 3 * c + x] = centers[3 * c + x];
        }
        upload(ctx->scratch_c, nuc, st);
        DeviceBuffer d_seg;
        upload(d_seg, seg_ao, st);
        ctx->scratch_b.reserve((size_t)n * n * sizeof(double2));
        ctx->reset_status();
        GX_CUDA(gx::launch_nuclear(b->dev(), pair_view(b, fp), ctx->boys(), ctx->t->gl.as<gx::GLRules>(),
                                   ctx->t->herm.as<uint32_t>(), b->d_classes.as<gx::PairClassDev>(),
                                   b->d_pp_class.as<int>(), nnuc, ctx->scratch_c.as<double>(),
                                   ctx->scratch_c.as<double>() + nnuc, d_seg.as<long long>(), n, 2 * lmax, nab_max,
                                   ctx->scratch_b.as<double2>(), ctx->status.as<gx::DevStatus>(), st));
        GX_CUDA(cudaMemcpyAsync(out, ctx->scratch_b.ptr, (size_t)n * n * sizeof(double2), cudaMemcpyDeviceToHost, st));
        GX_CUDA(cudaStreamSynchronize(st));
        check_status(ctx);
    });
}

int gx_cholesky_diagonal(gx_context* ctx, gx_basis* b, const int64_t* pairs, int64_t npairs, const double* B,
                         const double* O, double* out) {
    return guarded([&] {
        if (!ctx || !b) raise(GX_EINVAL, "null context or basis");
        check_field(B, O);
        const int ns = b->ns;
        const int64_t n = b->nao;
        std::vector<char> seen((size_t)ns * ns, 0);
        for (int64_t i = 0; i < npairs; ++i) {
            const int64_t a = pairs[2 * i], c = pairs[2 * i + 1];
            if (a < 0 || c < 0 || a >= ns || c >= ns || a > c)
                raise(GX_ERANGE, "Cholesky diagonal shell pair must be valid and ordered");
            if (seen[(size_t)a * ns + c]) raise(GX_EINVAL, "duplicate Cholesky diagonal shell pair");
            seen[(size_t)a * ns + c] = 1;
        }
        std::lock_guard<std::mutex> lock(ctx->mu);
        GX_CUDA(cudaSetDevice(ctx->device));
        std::vector<QuartetRequest> req;
        int64_t off = 0;
        for (int64_t i = 0; i < npairs; ++i) {
            const uint32_t a = (uint32_t)pairs[2 * i], c = (uint32_t)pairs[2 * i + 1];
            req.push_back({a, c, c, a, off});
            off += b->nao_of(a) * b->nao_of(c) * b->nao_of(c) * b->nao_of(a);
        }
        std::fill(out, out + n * n, 0.0);
        if (req.empty()) return;
        ctx->scratch_a.reserve(off * sizeof(double2));
        run_quartets(ctx, b, B, O, req, ctx->scratch_a.as<double2>(), nullptr);
        std::vector<std::complex<double>> host(off);
        GX_CUDA(cudaMemcpy(host.data(), ctx->scratch_a.ptr, off * sizeof(double2), cudaMemcpyDeviceToHost));
        for (const auto& r : req) {
            const int64_t na = b->nao_of(r.a), nb = b->nao_of(r.b);
            const std::complex<double>* blk = host.data() + r.out_off;
            for (int64_t i = 0; i < na; ++i)
                for (int64_t j = 0; j < nb; ++j) {
                    const double v = blk[((i * nb + j) * nb + j) * na + i].real();
                    const int64_t mu = b->ao_off[r.a] + i, nu = b->ao_off[r.b] + j;
                    out[nu * n + mu] = v;
                    if (r.a != r.b) out[mu * n + nu] = v;
                }
        }
    });
}

int gx_cholesky_columns(gx_context* ctx, gx_basis* b, const int64_t* pivots, int64_t npiv, const double* B,
                        const double* O, double* out) {
    return guarded([&] {
        if (!ctx || !b) raise(GX_EINVAL, "null context or basis");
        check_field(B, O);
        const int ns = b->ns;
        const int64_t n = b->nao;
        if (npiv == 0) return;
        std::vector<int> owner(n);
        for (int s = 0; s < ns; ++s)
            for (int64_t i = b->ao_off[s]; i < b->ao_off[s] + b->nao_of(s); ++i) owner[i] = s;
        for (int64_t k = 0; k < npiv; ++k)
            if (pivots[2 * k] < 0 || pivots[2 * k + 1] < 0 || pivots[2 * k] >= n || pivots[2 * k + 1] >= n)
                raise(GX_ERANGE, "Cholesky pivot AO index is out of range");
        const int sa = owner[pivots[0]], sb = owner[pivots[1]];
        for (int64_t k = 0; k < npiv; ++k)
            if (owner[pivots[2 * k]] != sa || owner[pivots[2 * k + 1]] != sb)
                raise(GX_EINVAL, "Cholesky candidate pivots must share a shell pair");
        const bool real = B[0] == 0.0 && B[1] == 0.0 && B[2] == 0.0;
        std::lock_guard<std::mutex> lock(ctx->mu);
        GX_CUDA(cudaSetDevice(ctx->device));
        std::vector<QuartetRequest> req;
        int64_t off = 0;
        for (int a = 0; a < ns; ++a)
            for (int c = real ? a : 0; c < ns; ++c) {
                req.push_back({(uint32_t)a, (uint32_t)c, (uint32_t)sb, (uint32_t)sa, off});
                off += b->nao_of(a) * b->nao_of(c) * b->nao_of(sb) * b->nao_of(sa);
            }
        ctx->scratch_a.reserve(off * sizeof(double2));
        run_quartets(ctx, b, B, O, req, ctx->scratch_a.as<double2>(), nullptr);
        std::vector<std::complex<double>> host(off);
        GX_CUDA(cudaMemcpy(host.data(), ctx->scratch_a.ptr, off * sizeof(double2), cudaMemcpyDeviceToHost));
        const int64_t nc = b->nao_of(sb), nd = b->nao_of(sa);
        for (const auto& r : req) {
            const int64_t na = b->nao_of(r.a), nb = b->nao_of(r.b);
            const std::complex<double>* blk = host.data() + r.out_off;
            for (int64_t k = 0; k < npiv; ++k) {
                const int64_t c = pivots[2 * k + 1] - b->ao_off[sb], d = pivots[2 * k] - b->ao_off[sa];
                for (int64_t i = 0; i < na; ++i)
                    for (int64_t j = 0; j < nb; ++j) {
                        const std::complex<double> v = blk[((i * nb + j) * nc + c) * nd + d];
                        const int64_t mu = b->ao_off[r.a] + i, nu = b->ao_off[r.b] + j;
                        if (real) {
                            double s = v.real();
                            if (r.a == r.b) s = (s + blk[((j * nb + i) * nc + c) * nd + d].real()) * 0.5;
                            out[(k * n + mu) * n + nu] = s;
                            if (r.a != r.b) out[(k * n + nu) * n + mu] = s;
                        } else {
                            out[2 * ((k * n + mu) * n + nu)] = v.real();
                            out[2 * ((k * n + mu) * n + nu) + 1] = v.imag();
                        }
                    }
            }
        }
    });
}

}  // extern "C"

namespace {

struct CholRed {
    double maxv;
    long long idx;
    double minv;
};

// Device column slots shared by the current candidate batch and the raw-column
// cache (python/giao_integrals/cholesky.py:180-265).
struct ColumnPool {
    DeviceBuffer buf;
    size_t col_bytes = 0;
    int capacity = 0;
    std::vector<int> refs, free_list;
    void init(int cap, size_t bytes) {
        capacity = cap;
        col_bytes = bytes;
        buf.reserve((size_t)cap * bytes);
        refs.assign(cap, 0);
        free_list.clear();
        for (int i = cap - 1; i >= 0; --i) free_list.push_back(i);
    }
    int take() {
        if (free_list.empty()) raise(GX_ENOMEM, "Cholesky column pool exhausted");
        const int s = free_list.back();
        free_list.pop_back();
        refs[s] = 1;
        return s;
    }
    void retain(int s) { ++refs[s]; }
    void release(int s) {
        if (--refs[s] == 0) free_list.push_back(s);
    }
    void* ptr(int s) const { return static_cast<char*>(buf.ptr) + (size_t)s * col_bytes; }
};

// Least-recently-inserted key set with the assignment semantics of a Python
// OrderedDict: inserting a present key keeps its position.
struct KeyOrder {
    std::list<int64_t> order;
    std::unordered_map<int64_t, std::list<int64_t>::iterator> pos;
    bool contains(int64_t k) const { return pos.count(k) != 0; }
    void insert(int64_t k) {
        if (!contains(k)) pos[k] = order.insert(order.end(), k);
    }
    void erase(int64_t k) {
        auto it = pos.find(k);
        if (it == pos.end()) return;
        order.erase(it->second);
        pos.erase(it);
    }
    void trim(size_t cap) {
        while (order.size() > cap) {
            pos.erase(order.front());
            order.pop_front();
        }
    }
};

}  // namespace

// Factors of one pivoted Cholesky, resident on the device until destroyed.
struct gx_cholesky_factors {
    gx_context* ctx = nullptr;
    DeviceBuffer L;              // rank rows of n*n (float64 on the real path, complex128 otherwise)
    int64_t cap_rows = 0;
    std::vector<int64_t> pivots;  // 2 * rank
    int64_t n = 0, rank = 0;
    bool real = false;
    double max_residual = 0.0;
    gx_cholesky_stats stats{};
};

namespace {

// Column evaluations replayed as CUDA graphs.  Pivot shell pairs of the
// same kind (angular momenta and primitive counts) give column plans of the
// same shape: the same classes, task counts and work units, only the task
// records differ.  One graph per shape and device view (the basis, pair
// records, tables and output it reads) runs the class launches on task and
// unit arrays of its own, which each evaluation refills from its plan (two
// device copies) before the replay: one launch instead of one per class, and
// no capture again for later factorisations of the same basis and field.
}  // namespace

struct ShapeGraph {
    PlanData plan;  // the shape's classes and units over buffers of its own
    DeviceBuffer counters;
    cudaGraphExec_t exec = nullptr;
    ~ShapeGraph() {
        if (exec) cudaGraphExecDestroy(exec);
    }
};

// Column evaluation of one pivot shell pair: its plan, block offsets and
// orientations, and primitive-quartet counters (accumulated over its
// evaluations when launched directly).
struct ColumnPlan {
    PlanData plan;
    DeviceBuffer boff, flip, counters;
    int nblocks = 0;
    int64_t entries = 0;
};

namespace {

constexpr size_t kMaxShapeGraphs = 256;
constexpr size_t kMaxColumnPlanBytes = size_t(1) << 30;

// Key of a column plan's graph: its shape and every address its launches read.
std::vector<long long> plan_shape(const PlanData& pd, const gx::EriDev& dev) {
    auto p = [](const void* x) { return (long long)(uintptr_t)x; };
    std::vector<long long> sig{(long long)pd.classes.size(), pd.ntask, (long long)pd.base.dev.bytes,
                               dev.basis.ns, p(dev.basis.center), p(dev.basis.l), p(dev.basis.nprim),
                               p(dev.basis.primoff), p(dev.basis.exps), p(dev.basis.coefs), p(dev.basis.raw),
                               p(dev.basis.sp_off), dev.pairs.npp, p(dev.pairs.p), p(dev.pairs.Pr),
                               p(dev.pairs.Pi), p(dev.pairs.F), p(dev.pairs.Eoff), p(dev.pairs.Epool),
                               p(dev.pairs.bound), p(dev.pairs.Epool32), p(dev.pairs.order), p(dev.pairs.sbound),
                               p(dev.pairs.g32), p(dev.boys.S), p(dev.boys.E0), p(dev.gl), p(dev.herm_xyz),
                               p(dev.rec_plan), p(dev.rec_plan_off), p(dev.out), p(dev.status)};
    uint32_t cuts[2];
    std::memcpy(&cuts[0], &dev.skip_cut, 4);
    std::memcpy(&cuts[1], &dev.fp32_cut, 4);
    sig.push_back(cuts[0]);
    sig.push_back(cuts[1]);
    for (size_t ci = 0; ci < pd.classes.size(); ++ci) {
        const auto& pc = pd.classes[ci];
        sig.insert(sig.end(), {pc.key[0], pc.key[1], pc.key[2], pc.key[3], (long long)pc.first, (long long)pc.count,
                               (long long)pd.base.range[ci].first, (long long)pd.base.range[ci].second,
                               (long long)pd.base.lane[ci].first, (long long)pd.base.lane[ci].second});
    }
    return sig;
}

// The pivot loop of python/giao_integrals/cholesky.py:60-297 on the device:
// residual diagonal, argmax (lowest flat index on ties), column generation,
// factor update and PSD check stay resident; the host sees one reduction
// record per pivot.  The factor rows grow in f.L (doubling) up to `limit`.
void cholesky_core(gx_context* ctx, gx_basis* b, const double* Bf, const double* Of, const gx_cholesky_options* opt,
                   gx_cholesky_factors& f) {
    const auto wall0 = std::chrono::steady_clock::now();
    const double threshold = opt->threshold, screening = opt->screening_threshold;
    if (!std::isfinite(threshold) || threshold < 0.0) raise(GX_EINVAL, "threshold must be finite and non-negative");
    if (!std::isfinite(screening) || screening < 0.0)
        raise(GX_EINVAL, "screening_threshold must be finite and non-negative");
    if (opt->pivot_batch_size < 1) raise(GX_EINVAL, "pivot_batch_size must be a positive integer");
    GX_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    const int ns = b->ns;
    const int64_t n = b->nao, N = n * n;
    gx_cholesky_stats& stats = f.stats;
    stats = gx_cholesky_stats{};
    f.ctx = ctx;
    f.n = n;
    f.rank = 0;
    f.max_residual = 0.0;
    f.pivots.clear();
    if (n == 0) return;
    // single centre: the London phase cancels; use zero-field integrals (cholesky.py:130-133)
    bool single = true;
    for (int s = 1; s < ns; ++s)
        for (int k = 0; k < 3; ++k) single = single && b->center[3 * s + k] == b->center[k];
    const double zero3[3] = {0.0, 0.0, 0.0};
    const double* iB = single ? zero3 : Bf;
    const double* iO = single ? zero3 : Of;
    const bool real = (Bf[0] == 0.0 && Bf[1] == 0.0 && Bf[2] == 0.0) || single;
    f.real = real;
    const size_t esz = real ? sizeof(double) : sizeof(double2);
    std::vector<int> owner(n);
    for (int s = 0; s < ns; ++s)
        for (int64_t i = b->ao_off[s]; i < b->ao_off[s] + b->nao_of(s); ++i) owner[i] = s;

    // event timing of the column evaluations and of the factor update
    struct EventPair {
        cudaEvent_t a = nullptr, b = nullptr;
        ~EventPair() {
            if (a) cudaEventDestroy(a);
            if (b) cudaEventDestroy(b);
        }
    } ev_col, ev_upd;
    GX_CUDA(cudaEventCreate(&ev_col.a));
    GX_CUDA(cudaEventCreate(&ev_col.b));
    GX_CUDA(cudaEventCreate(&ev_upd.a));
    GX_CUDA(cudaEventCreate(&ev_upd.b));
    bool col_pending = false, upd_pending = false;
    auto collect_times = [&] {  // after a stream synchronisation
        float ms = 0.0f;
        if (col_pending) {
            GX_CUDA(cudaEventElapsedTime(&ms, ev_col.a, ev_col.b));
            stats.column_ms += ms;
            col_pending = false;
        }
        if (upd_pending) {
            GX_CUDA(cudaEventElapsedTime(&ms, ev_upd.a, ev_upd.b));
            stats.update_ms += ms;
            upd_pending = false;
        }
    };

    // ---- diagonal (with optional Schwarz skip of initial blocks) ----
    DeviceBuffer d_D, d_res, d_partial, d_red, d_scale, d_work, d_boff, d_info, d_cand, d_dst;
    d_D.reserve(N * sizeof(double));
    d_res.reserve(N * sizeof(double));
    d_partial.reserve(gx::chol_partial_bytes());
    d_red.reserve(gx::chol_red_bytes());
    d_scale.reserve(sizeof(double));
    GX_CUDA(cudaMemsetAsync(d_D.ptr, 0, N * sizeof(double), st));
    std::vector<double> q;
    if (screening > 0.0) q = schwarz_values(ctx, b, iB, iO);
    std::vector<std::pair<int, int>> measured, skipped;
    std::vector<double> skip_fill;
    for (int a = 0; a < ns; ++a)
        for (int c = a; c < ns; ++c) {
            const double qq = screening > 0.0 ? q[(size_t)a * ns + c] * q[(size_t)a * ns + c] : 0.0;
            if (screening > 0.0 && qq <= std::min(threshold, screening)) {
                skipped.push_back({a, c});
                skip_fill.push_back(qq);
            } else {
                measured.push_back({a, c});
            }
        }
    auto read_diagonal = [&](const std::vector<std::pair<int, int>>& pairs, double* target) {
        if (pairs.empty()) return;
        std::vector<QuartetRequest> req;
        std::vector<long long> boff;
        std::vector<int> info;
        int64_t off = 0;
        for (const auto& pr : pairs) {
            const uint32_t a = pr.first, c = pr.second;
            req.push_back({a, c, c, a, off});
            boff.push_back(off);
            info.insert(info.end(), {(int)b->ao_off[a], (int)b->ao_off[c], (int)b->nao_of(a), (int)b->nao_of(c)});
            off += b->nao_of(a) * b->nao_of(c) * b->nao_of(c) * b->nao_of(a);
        }
        ctx->scratch_a.reserve(off * sizeof(double2));
        PlanData dplan;
        build_plan(ctx, b, req, dplan);
        int64_t evaluated[2] = {0, 0};
        run_plan(ctx, b, iB, iO, dplan, ctx->scratch_a.as<double2>(), nullptr, nullptr, GX_PRECISION_FP64, 0.0,
                 evaluated);
        stats.diagonal_primitive_quartets += evaluated[0];
        upload(d_boff, boff, st);
        upload(d_info, info, st);
        GX_CUDA(gx::launch_chol_diag(ctx->scratch_a.as<double2>(), d_boff.as<long long>(), d_info.as<int>(),
                                     (int)pairs.size(), (int)n, target, st));
    };
    read_diagonal(measured, d_D.as<double>());
    if (!skipped.empty()) {
        std::vector<double> D(N);
        GX_CUDA(cudaMemcpyAsync(D.data(), d_D.ptr, N * sizeof(double), cudaMemcpyDeviceToHost, st));
        GX_CUDA(cudaStreamSynchronize(st));
        for (size_t k = 0; k < skipped.size(); ++k) {
            const int a = skipped[k].first, c = skipped[k].second;
            for (int64_t i = b->ao_off[a]; i < b->ao_off[a] + b->nao_of(a); ++i)
                for (int64_t j = b->ao_off[c]; j < b->ao_off[c] + b->nao_of(c); ++j) {
                    D[i * n + j] = skip_fill[k];
                    D[j * n + i] = skip_fill[k];
                }
        }
        GX_CUDA(cudaMemcpyAsync(d_D.ptr, D.data(), N * sizeof(double), cudaMemcpyHostToDevice, st));
    }
    GX_CUDA(cudaMemcpyAsync(d_res.ptr, d_D.ptr, N * sizeof(double), cudaMemcpyDeviceToDevice, st));
    CholRed red;
    int status_code = 0;
    // page-locked mailbox of the loop's small transfers (asynchronous both ways)
    constexpr int kMailLog = 256;
    struct Mail {
        gx::ChainState cs_in, cs_out;
        CholRed red;
        int status, pad;
        long long log[kMailLog];
    };
    ctx->chol_mail.reserve(sizeof(Mail));
    Mail* mail = static_cast<Mail*>(ctx->chol_mail.p);
    auto fetch_red = [&] {
        // the reduction result and the kernels' status word in one wait (a
        // failure in a column batch is reported before the next pivot)
        GX_CUDA(cudaMemcpyAsync(&mail->red, d_red.ptr, sizeof(CholRed), cudaMemcpyDeviceToHost, st));
        GX_CUDA(cudaMemcpyAsync(&mail->status, ctx->status.ptr, sizeof(int), cudaMemcpyDeviceToHost, st));
        GX_CUDA(cudaStreamSynchronize(st));
        red = mail->red;
        status_code = mail->status;
        collect_times();
        if (status_code) check_status(ctx);
    };
    GX_CUDA(gx::launch_chol_scan(d_res.as<double>(), N, d_partial.ptr, d_red.ptr, st));
    fetch_red();
    const double floor = 64 * 2.220446049250313e-16 * std::max(red.maxv, 0.0);
    const double tol = std::max(threshold, floor);
    const int64_t limit = std::min<int64_t>(N, opt->max_rank);

    // ---- pivot loop ----
    bool reuse = !single;
    for (int s = 0; s < ns; ++s) reuse = reuse || b->ncontr[s] > 1 || b->nprim[s] > 1;
    // The local block rule of complex contracted systems (cholesky.py:195-206).
    // Its candidates are the contraction variants of an evaluated pivot; with
    // one contraction per shell that is the pivot alone, whose residual is
    // zero once taken, so the rule never overrides the global argmax.
    bool general = false;
    for (int s = 0; s < ns; ++s) general = general || b->ncontr[s] > 1;
    const bool local_rule = reuse && !real && opt->pivot_batch_size > 1 && general;
    // Columns kept per pivot-block evaluation: the evaluation computes every
    // column of the pivot's shell-pair block, and raw columns are exact
    // whenever they are computed, so keeping more of them (and the raw-column
    // cache below) changes only how often a block is evaluated.  Pivots are
    // decided by the reference's own candidate and cache state, tracked
    // separately (ref_* below) when its local rule is in force.
    constexpr int kBatchColumns = 256;
    const size_t col_bytes = N * esz;
    int cache_cap = 1024;
    {
        // the raw-column cache only saves re-evaluations: fit it into half of
        // the free device memory left after the first factor rows
        size_t free_b = 0, total_b = 0;
        GX_CUDA(cudaMemGetInfo(&free_b, &total_b));
        const int64_t first_rows = std::min<int64_t>(std::max<int64_t>(limit, 1), std::max<int64_t>(64, 8 * n));
        const double room = (double)free_b * 0.5 - (double)first_rows * col_bytes - 8.0 * col_bytes;
        const int64_t fit = (int64_t)(room / (double)col_bytes) - kBatchColumns - 64;
        cache_cap = (int)std::max<int64_t>(0, std::min<int64_t>(2048, fit));
    }
    ColumnPool pool;
    pool.init(kBatchColumns + cache_cap + 64, col_bytes);
    stats.column_cache_capacity = cache_cap;
    // Chained steps (no local block rule): the device takes the next pivots
    // itself while their raw columns are cached; slot_of mirrors the cache.
    const bool chain_ok = !local_rule;
    DeviceBuffer d_slot_of, d_state, d_log;
    std::vector<int> slot_of_h;
    bool slot_dirty = true;
    int chain_k = 8;
    slot_of_h.assign(N, -1);  // cache slot of every flat index (-1: not cached)
    if (chain_ok) {
        d_slot_of.reserve(N * sizeof(int));
        d_state.reserve(sizeof(gx::ChainState));
        d_log.reserve(std::max<int64_t>(limit, 1) * sizeof(long long));
        ctx->chol_slots.reserve(N * sizeof(int));
    }
    struct GraphSet {  // instantiated chain graphs, destroyed with the factorisation
        std::map<std::tuple<int, void*, int>, cudaGraphExec_t> m;
        ~GraphSet() {
            for (auto& kv : m) cudaGraphExecDestroy(kv.second);
        }
    } chain_graph_set;
    auto& chain_graphs = chain_graph_set.m;
    auto set_slot = [&](int64_t fl, int v) {
        slot_of_h[fl] = v;
        slot_dirty = true;
    };
    d_work.reserve(col_bytes);
    constexpr int kGemvChunks = 8;  // rank chunks of the factor update (partial sums)
    DeviceBuffer d_gemv;
    d_gemv.reserve((size_t)kGemvChunks * col_bytes);
    f.cap_rows = std::min<int64_t>(std::max<int64_t>(limit, 1), std::max<int64_t>(64, 8 * n));
    f.L.reserve((size_t)f.cap_rows * col_bytes);
    std::vector<int64_t> cands;               // current batch candidates (flat indices)
    std::vector<int> cand_slot;               // their column slots
    std::list<std::pair<int64_t, int>> lru;   // raw-column cache, oldest first
    std::map<int64_t, std::list<std::pair<int64_t, int>>::iterator> lru_pos;
    // the reference's candidate batch, block candidates and raw-column cache keys
    std::vector<int64_t> ref_cands, block_cands;
    KeyOrder ref_cache;
    std::vector<double> hostblk;
    // the context's column plans this factorisation used (held) and their
    // counters when it began
    std::map<ColumnPlan*, std::pair<std::shared_ptr<ColumnPlan>, std::vector<unsigned long long>>> plan_base;
    DeviceBuffer column_info;
    // Column evaluations replayed as CUDA graphs (ShapeGraph), cached in the
    // context across factorisations.
    auto& shape_graphs = ctx->shape_graphs;
    // the graphs this factorisation replayed (held, so that clearing the
    // context's cache cannot free them) and their counters when it began
    std::map<ShapeGraph*, std::pair<std::shared_ptr<ShapeGraph>, std::vector<unsigned long long>>> shape_base;
    {
        // largest column batch: all (x, y) blocks against the largest pivot pair
        int64_t sum_xy = 0, max_ao = 0;
        for (int x = 0; x < ns; ++x) {
            max_ao = std::max<int64_t>(max_ao, b->nao_of(x));
            for (int y = real ? x : 0; y < ns; ++y) sum_xy += b->nao_of(x) * b->nao_of(y);
        }
        ctx->scratch_a.reserve(std::max<int64_t>(sum_xy * max_ao * max_ao, 1) * sizeof(double2));
    }
    int64_t rank = 0;
    auto residual_at = [&](const std::vector<int64_t>& idx, std::vector<double>& vals) {
        vals.resize(idx.size());
        for (size_t k = 0; k < idx.size(); ++k)
            GX_CUDA(cudaMemcpyAsync(&vals[k], d_res.as<double>() + idx[k], sizeof(double), cudaMemcpyDeviceToHost,
                                    st));
        GX_CUDA(cudaStreamSynchronize(st));
    };
    auto drop_batch = [&] {
        for (int s : cand_slot) pool.release(s);
        cands.clear();
        cand_slot.clear();
    };
    // Residual of the pivot's shell-pair block on the host (one strided 2-D
    // copy) and the reference's candidate list: the contraction variants of
    // the pivot (reuse) or the whole block, above the tolerance, largest
    // residual first (stable), at most `count`, the pivot forced in
    // (cholesky.py:225-242).
    int blk_a = -1, blk_c = -1;
    int64_t blk_rank = -1;
    auto load_block = [&](int64_t pivot) {
        const int64_t mu = pivot / n, nu = pivot % n;
        const int a = owner[mu], c = owner[nu];
        if (a == blk_a && c == blk_c && blk_rank == rank) return;
        const int64_t na = b->nao_of(a), nc = b->nao_of(c);
        hostblk.resize(na * nc);
        GX_CUDA(cudaMemcpy2DAsync(hostblk.data(), nc * sizeof(double),
                                  d_res.as<double>() + b->ao_off[a] * n + b->ao_off[c], n * sizeof(double),
                                  nc * sizeof(double), na, cudaMemcpyDeviceToHost, st));
        GX_CUDA(cudaStreamSynchronize(st));
        blk_a = a;
        blk_c = c;
        blk_rank = rank;
    };
    auto rv = [&](int64_t f_) {
        return hostblk[(f_ / n - b->ao_off[blk_a]) * b->nao_of(blk_c) + (f_ % n - b->ao_off[blk_c])];
    };
    auto reference_candidates = [&](int64_t pivot, int count) {
        load_block(pivot);
        const int a = blk_a, c = blk_c;
        const int64_t mu = pivot / n, nu = pivot % n;
        std::vector<int64_t> idx;
        if (reuse) {
            const int ca = b->ncart_of(a), cc = b->ncart_of(c);
            for (int xa = 0; xa < b->ncontr[a]; ++xa)
                for (int xc = 0; xc < b->ncontr[c]; ++xc)
                    idx.push_back((b->ao_off[a] + (mu - b->ao_off[a]) % ca + (int64_t)ca * xa) * n + b->ao_off[c] +
                                  (nu - b->ao_off[c]) % cc + (int64_t)cc * xc);
        } else {
            for (int64_t i = b->ao_off[a]; i < b->ao_off[a] + b->nao_of(a); ++i)
                for (int64_t j = b->ao_off[c]; j < b->ao_off[c] + b->nao_of(c); ++j) idx.push_back(i * n + j);
        }
        std::vector<int64_t> keep;
        for (int64_t x : idx)
            if (rv(x) > tol) keep.push_back(x);
        std::stable_sort(keep.begin(), keep.end(), [&](int64_t x, int64_t y) { return rv(x) > rv(y); });
        if ((int)keep.size() > count) keep.resize(count);
        if (std::find(keep.begin(), keep.end(), pivot) == keep.end()) {
            if (keep.empty())
                keep.push_back(pivot);
            else
                keep.back() = pivot;
        }
        return keep;
    };
    while (red.maxv > tol) {
        int64_t pivot = red.idx;
        if (local_rule && !block_cands.empty()) {
            std::vector<double> v;
            residual_at(block_cands, v);
            size_t best = 0;
            for (size_t k = 1; k < v.size(); ++k)
                if (v[k] > v[best]) best = k;
            if (v[best] > tol && v[best] >= 0.01 * red.maxv) pivot = block_cands[best];
        }
        if (rank >= limit) {
            f.rank = rank;
            stats.rank = rank;
            raise(GX_ENOMEM, "Cholesky rank capacity exceeded");
        }
        if (rank >= f.cap_rows || (chain_ok && rank + 1 + chain_k > f.cap_rows && f.cap_rows < limit)) {
            // grow the factor rows (doubling, at most `limit`)
            const int64_t cap2 = std::min<int64_t>(limit, std::max<int64_t>(2 * f.cap_rows, rank + 1 + chain_k));
            DeviceBuffer grown;
            grown.reserve((size_t)cap2 * col_bytes);
            GX_CUDA(cudaMemcpyAsync(grown.ptr, f.L.ptr, (size_t)rank * col_bytes, cudaMemcpyDeviceToDevice, st));
            GX_CUDA(cudaStreamSynchronize(st));
            std::swap(grown.ptr, f.L.ptr);
            std::swap(grown.bytes, f.L.bytes);
            f.cap_rows = cap2;
        }
        // The reference's state decides the local rule's candidates: a pivot
        // found in its raw-column cache replaces its batch by the pivot alone;
        // a pivot outside its batch makes it evaluate the pivot's block, whose
        // contraction variants become the block candidates and enter its cache
        // (capacity min(1024, max(8, rank + 8))).
        if (local_rule) {
            if (ref_cache.contains(pivot)) {
                ref_cands.assign(1, pivot);
                ref_cache.erase(pivot);
            }
            if (std::find(ref_cands.begin(), ref_cands.end(), pivot) == ref_cands.end()) {
                ref_cands = reference_candidates(pivot, 32);
                block_cands.assign(ref_cands.begin(),
                                   ref_cands.begin() + std::min<size_t>(ref_cands.size(),
                                                                        std::min(32, opt->pivot_batch_size)));
                for (int64_t x : ref_cands)
                    if (x != pivot) ref_cache.insert(x);
                ref_cache.trim((size_t)std::min<int64_t>(1024, std::max<int64_t>(8, rank + 8)));
            }
            ref_cache.erase(pivot);
        }
        // Physical supply of the raw column: the current batch, the raw-column
        // cache, or a new evaluation of the pivot's block.
        auto cached = lru_pos.find(pivot);
        if (cached != lru_pos.end() &&
            std::find(cands.begin(), cands.end(), pivot) == cands.end()) {
            const int slot = cached->second->second;
            lru.erase(cached->second);
            lru_pos.erase(cached);
            set_slot(pivot, -1);
            drop_batch();
            cands.push_back(pivot);
            cand_slot.push_back(slot);  // cache reference moves to the batch
        }
        auto it = std::find(cands.begin(), cands.end(), pivot);
        if (it == cands.end()) {
            const int64_t mu = pivot / n, nu = pivot % n;
            const int a = owner[mu], c = owner[nu];
            std::vector<int64_t> keep = reference_candidates(pivot, reuse ? 32 : kBatchColumns);
            {
                // the evaluation computes every column of the block: keep the
                // other entries above the threshold too (largest residual
                // first) for the raw-column cache
                std::vector<int64_t> extra;
                const int64_t na = b->nao_of(a), nc = b->nao_of(c);
                for (int64_t i = b->ao_off[a]; i < b->ao_off[a] + na; ++i)
                    for (int64_t j = b->ao_off[c]; j < b->ao_off[c] + nc; ++j) {
                        const int64_t fl = i * n + j;
                        if (rv(fl) > tol && std::find(keep.begin(), keep.end(), fl) == keep.end()) extra.push_back(fl);
                    }
                std::stable_sort(extra.begin(), extra.end(), [&](int64_t x, int64_t y) { return rv(x) > rv(y); });
                const size_t room = keep.size() < (size_t)kBatchColumns ? kBatchColumns - keep.size() : 0;
                if (extra.size() > room) extra.resize(room);
                keep.insert(keep.end(), extra.begin(), extra.end());
            }
            drop_batch();
            cands = keep;
            // The pivot's block.  (Evaluating the blocks of the next largest
            // uncached residual entries in the same launches was measured:
            // 2-4 blocks per evaluation cost more column time than they saved
            // on both the 140-AO atom and the 12-atom molecule.)
            struct EvalBlock {
                int sa, sb;
                std::vector<int64_t> cols;
            };
            std::vector<EvalBlock> blocks{{a, c, {}}};
            blocks[0].cols = cands;
            // columns (mu nu | p1 p0) for all shell pairs (real: b >= a).  The
            // quartet list, its plan and block offsets depend only on the
            // pivot shell pair: built once per factorisation and reused.
            std::vector<ColumnPlan*> cps;
            std::vector<int64_t> sbase;
            int64_t stot = 0;
            for (const auto& bl : blocks) {
                const int sa = bl.sa, sb = bl.sb;
                const auto pkey = std::make_tuple(static_cast<const gx_basis*>(b), sa, sb, real);
                if (ctx->column_plan_bytes > kMaxColumnPlanBytes && !ctx->column_plans.count(pkey)) {
                    ctx->column_plans.clear();  // (the plans in use here are held by plan_base)
                    ctx->column_plan_bytes = 0;
                }
                auto& cp = ctx->column_plans[pkey];
                if (!cp) {
                    cp = std::make_shared<ColumnPlan>();
                    std::vector<QuartetRequest> req;
                    std::vector<long long> boff;
                    std::vector<int> flip;
                    int64_t off = 0;
                    // (x y | sb sa), or (sb sa | x y) when (x, y) has the
                    // higher angular momentum and at least as many primitive
                    // pairs: the kernels spread the ket components of a shell
                    // quartet over warps, so the wide pair goes to the ket (a
                    // low-L pivot against high-L bra pairs otherwise leaves a
                    // few warps on the long tasks), but they contract each
                    // bra primitive pair once over all its ket primitive
                    // pairs, so a contracted pivot pair stays in the ket (on
                    // the 12-atom molecule, flipping against contracted s
                    // pivots made the column evaluations 18% slower)
                    const int lpiv = b->l[sa] + b->l[sb];
                    const int kpiv = b->nprim[sa] * b->nprim[sb];
                    for (int x = 0; x < ns; ++x)
                        for (int y = real ? x : 0; y < ns; ++y) {
                            const bool fl = b->l[x] + b->l[y] > lpiv && b->nprim[x] * b->nprim[y] >= kpiv;
                            if (fl)
                                req.push_back({(uint32_t)sb, (uint32_t)sa, (uint32_t)x, (uint32_t)y, off});
                            else
                                req.push_back({(uint32_t)x, (uint32_t)y, (uint32_t)sb, (uint32_t)sa, off});
                            boff.push_back(off);
                            flip.push_back(fl ? 1 : 0);
                            off += b->nao_of(x) * b->nao_of(y) * b->nao_of(sb) * b->nao_of(sa);
                        }
                    build_plan(ctx, b, req, cp->plan);
                    upload(cp->boff, boff, st);
                    upload(cp->flip, flip, st);
                    cp->nblocks = (int)req.size();
                    cp->entries = off;
                    cp->counters.reserve(std::max<size_t>(2 * cp->plan.classes.size(), 2) *
                                         sizeof(unsigned long long));
                    GX_CUDA(cudaMemsetAsync(cp->counters.ptr, 0, cp->counters.bytes, st));
                    ctx->column_plan_bytes += cp->plan.tasks.bytes + cp->plan.base.dev.bytes + cp->boff.bytes;
                }
                if (!plan_base.count(cp.get())) {
                    std::vector<unsigned long long> c(2 * cp->plan.classes.size());
                    if (!c.empty()) {
                        GX_CUDA(cudaMemcpyAsync(c.data(), cp->counters.ptr, c.size() * sizeof(unsigned long long),
                                                cudaMemcpyDeviceToHost, st));
                        GX_CUDA(cudaStreamSynchronize(st));
                    }
                    plan_base.emplace(cp.get(), std::make_pair(cp, std::move(c)));
                }
                cps.push_back(cp.get());
                sbase.push_back(stot);
                stot += cp->entries;
            }
            ctx->scratch_a.reserve(std::max<int64_t>(stot, 1) * sizeof(double2));
            if (column_info.ptr == nullptr) {
                std::vector<int> info;
                for (int x = 0; x < ns; ++x)
                    for (int y = real ? x : 0; y < ns; ++y)
                        info.insert(info.end(), {(int)b->ao_off[x], (int)b->ao_off[y], (int)b->nao_of(x),
                                                 (int)b->nao_of(y), x == y ? 1 : 0});
                upload(column_info, info, st);
            }
            std::vector<int> cl;
            std::vector<void*> dst;
            std::vector<std::vector<int>> bslots(blocks.size());
            for (size_t k = 0; k < blocks.size(); ++k)
                for (int64_t fl : blocks[k].cols) {
                    cl.push_back((int)(fl % n - b->ao_off[blocks[k].sb]));  // c: p1 within sb
                    cl.push_back((int)(fl / n - b->ao_off[blocks[k].sa]));  // d: p0 within sa
                    const int slot = pool.take();
                    bslots[k].push_back(slot);
                    dst.push_back(pool.ptr(slot));
                }
            cand_slot = bslots[0];
            upload(d_cand, cl, st);
            upload(d_dst, dst, st);
            GX_CUDA(cudaEventRecord(ev_col.a, st));
            {
                // the blocks' class launches share one fork/join over the
                // auxiliary streams, so they fill the GPU together
                std::vector<std::pair<const PlanData*, gx::EriDev>> runs;
                FieldPairs& fpairs = field_pairs(b, iB, iO);
                for (size_t k = 0; k < blocks.size(); ++k)
                    runs.push_back({&cps[k]->plan, make_dev(ctx, b, fpairs, ctx->scratch_a.as<double2>() + sbase[k],
                                                            GX_PRECISION_FP64, 0.0)});
                std::vector<unsigned long long*> ctr;
                for (auto* cp : cps) ctr.push_back(cp->counters.as<unsigned long long>());
                // (the legacy default stream cannot be captured: launch directly there)
                const bool capturable = st != nullptr && st != cudaStreamLegacy && st != cudaStreamPerThread;
                const PlanData& pd = cps[0]->plan;
                if (blocks.size() == 1 && capturable && pd.ntask > 0) {
                    const auto key = plan_shape(pd, runs[0].second);
                    if (shape_graphs.size() >= kMaxShapeGraphs && !shape_graphs.count(key)) shape_graphs.clear();
                    auto& sg = shape_graphs[key];
                    if (!sg) {
                        sg = std::make_shared<ShapeGraph>();
                        PlanData& sp = sg->plan;
                        sp.classes = pd.classes;
                        sp.defconf = pd.defconf;
                        sp.order = pd.order;
                        sp.stable = pd.stable;
                        sp.ntask = pd.ntask;
                        sp.spread_parts = pd.spread_parts;
                        sp.base.range = pd.base.range;
                        sp.base.lane = pd.base.lane;
                        sp.tasks.reserve(pd.tasks.bytes);
                        sp.base.dev.reserve(pd.base.dev.bytes);
                        sg->counters.reserve(std::max<size_t>(2 * pd.classes.size(), 2) * sizeof(unsigned long long));
                        GX_CUDA(cudaMemsetAsync(sg->counters.ptr, 0, sg->counters.bytes, st));
                        cudaGraph_t graph = nullptr;
                        GX_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
                        try {
                            enqueue_plans(ctx, {{&sp, runs[0].second}}, GX_PRECISION_FP64,
                                          {sg->counters.as<unsigned long long>()});
                        } catch (...) {
                            cudaStreamEndCapture(st, &graph);
                            if (graph) cudaGraphDestroy(graph);
                            throw;
                        }
                        GX_CUDA(cudaStreamEndCapture(st, &graph));
                        const cudaError_t ie = cudaGraphInstantiate(&sg->exec, graph, 0);
                        cudaGraphDestroy(graph);
                        GX_CUDA(ie);
                    }
                    GX_CUDA(cudaMemcpyAsync(sg->plan.tasks.ptr, pd.tasks.ptr, sizeof(gx::Task) * pd.ntask,
                                            cudaMemcpyDeviceToDevice, st));
                    GX_CUDA(cudaMemcpyAsync(sg->plan.base.dev.ptr, pd.base.dev.ptr, pd.base.dev.bytes,
                                            cudaMemcpyDeviceToDevice, st));
                    if (!shape_base.count(sg.get())) {
                        // the counters accumulate across factorisations: note where this one starts
                        std::vector<unsigned long long> c(2 * pd.classes.size());
                        GX_CUDA(cudaMemcpyAsync(c.data(), sg->counters.ptr, c.size() * sizeof(unsigned long long),
                                                cudaMemcpyDeviceToHost, st));
                        GX_CUDA(cudaStreamSynchronize(st));
                        shape_base.emplace(sg.get(), std::make_pair(sg, std::move(c)));
                    }
                    GX_CUDA(cudaGraphLaunch(sg->exec, st));
                } else {
                    enqueue_plans(ctx, runs, GX_PRECISION_FP64, ctr);
                }
            }
            int64_t coff = 0;
            for (size_t k = 0; k < blocks.size(); ++k) {
                const int ncand = (int)blocks[k].cols.size();
                if (ncand)
                    GX_CUDA(gx::launch_chol_cols(real, ctx->scratch_a.as<double2>() + sbase[k], cps[k]->boff.as<long long>(),
                                                 column_info.as<int>(), cps[k]->flip.as<int>(), cps[k]->nblocks,
                                                 d_cand.as<int>() + 2 * coff,
                                                 ncand, (int)b->nao_of(blocks[k].sb), (int)b->nao_of(blocks[k].sa),
                                                 (int)n, d_dst.as<void*>() + coff, st));
                coff += ncand;
            }
            GX_CUDA(cudaEventRecord(ev_col.b, st));
            col_pending = true;
            ++stats.block_evaluations;
            stats.column_entries += (int64_t)coff * N;
            for (size_t k = 0; k < blocks.size(); ++k)
                for (size_t t = 0; t < blocks[k].cols.size(); ++t) {
                    const int64_t fl = blocks[k].cols[t];
                    const int sl = bslots[k][t];
                    if (k == 0 && fl == pivot) continue;
                    // assignment to an existing key keeps its position (OrderedDict semantics)
                    auto old = lru_pos.find(fl);
                    pool.retain(sl);
                    if (old != lru_pos.end()) {
                        pool.release(old->second->second);
                        old->second->second = sl;
                    } else {
                        lru.push_back({fl, sl});
                        lru_pos[fl] = std::prev(lru.end());
                    }
                    set_slot(fl, sl);
                }
            while (lru.size() > (size_t)cache_cap) {
                pool.release(lru.front().second);
                set_slot(lru.front().first, -1);
                lru_pos.erase(lru.front().first);
                lru.pop_front();
            }
            it = std::find(cands.begin(), cands.end(), pivot);
        }
        {
            auto c2it = lru_pos.find(pivot);
            if (c2it != lru_pos.end()) {
                pool.release(c2it->second->second);
                lru.erase(c2it->second);
                lru_pos.erase(c2it);
                set_slot(pivot, -1);
            }
        }
        const int slot = cand_slot[it - cands.begin()];
        void* Lrow = static_cast<char*>(f.L.ptr) + (size_t)rank * col_bytes;
        GX_CUDA(cudaEventRecord(ev_upd.a, st));
        GX_CUDA(gx::launch_chol_step(real, f.L.ptr, N, (int)rank, pivot, pool.ptr(slot), d_work.ptr, (int)n,
                                     d_res.as<double>(), d_scale.as<double>(), Lrow, d_partial.ptr, d_red.ptr, st,
                                     d_gemv.ptr, kGemvChunks, ctx->sm_count));
        const double psd = std::max(floor * 16, 1e-12);
        // then up to chain_k steps the device takes on its own while the next
        // pivot's raw column is cached (one host synchronisation for all)
        const bool chained = chain_ok && !lru.empty() && rank + 1 < std::min<int64_t>(limit, f.cap_rows);
        gx::ChainState cs_out{};
        std::vector<long long> chain_log;
        int64_t nlog = 0;
        if (chained) {
            if (slot_dirty) {
                // (the previous upload from the staging copy ended with the
                // previous iteration's synchronisation)
                std::memcpy(ctx->chol_slots.p, slot_of_h.data(), N * sizeof(int));
                GX_CUDA(cudaMemcpyAsync(d_slot_of.ptr, ctx->chol_slots.p, N * sizeof(int), cudaMemcpyHostToDevice,
                                        st));
                slot_dirty = false;
            }
            gx::ChainState cs{};
            cs.slot = -1;
            cs.rank = (int)rank + 1;
            cs.active = 1;
            cs.rank_limit = (int)std::min<int64_t>(limit, f.cap_rows);
            mail->cs_in = cs;
            GX_CUDA(cudaMemcpyAsync(d_state.ptr, &mail->cs_in, sizeof cs, cudaMemcpyHostToDevice, st));
            // the chain's launches replayed as one CUDA graph per (length,
            // factor buffer, rank-chunk count): one launch instead of three per step
            const int rank_hi = (int)rank + 1 + chain_k;
            const int nblk = (int)((N + 127) / 128);
            // (fixed once the rank reaches 64, so that few graphs are captured)
            const int nchunks =
                rank_hi >= 64 ? std::max(1, std::min(kGemvChunks, (8 * ctx->sm_count) / std::max(nblk, 1))) : 1;
            const auto gkey = std::make_tuple(chain_k, f.L.ptr, nchunks);
            // (the legacy default stream cannot be captured: launch directly there)
            const bool capturable = st != nullptr && st != cudaStreamLegacy && st != cudaStreamPerThread;
            auto git = chain_graphs.find(gkey);
            if (!capturable) {
                GX_CUDA(gx::launch_chol_chain(real, f.L.ptr, N, (int)n, rank_hi, chain_k,
                                              d_state.as<gx::ChainState>(), d_slot_of.as<int>(),
                                              d_log.as<long long>(), pool.buf.ptr, d_res.as<double>(),
                                              d_partial.ptr, d_red.ptr, d_gemv.ptr, kGemvChunks, ctx->sm_count, tol,
                                              psd, st));
            } else if (git == chain_graphs.end()) {
                cudaGraph_t graph = nullptr;
                GX_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
                const cudaError_t le = gx::launch_chol_chain(
                    real, f.L.ptr, N, (int)n, rank_hi, chain_k, d_state.as<gx::ChainState>(), d_slot_of.as<int>(),
                    d_log.as<long long>(), pool.buf.ptr, d_res.as<double>(), d_partial.ptr, d_red.ptr, d_gemv.ptr,
                    kGemvChunks, ctx->sm_count, tol, psd, st);
                const cudaError_t ce = cudaStreamEndCapture(st, &graph);
                GX_CUDA(le);
                GX_CUDA(ce);
                cudaGraphExec_t exec = nullptr;
                const cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
                cudaGraphDestroy(graph);
                GX_CUDA(ie);
                git = chain_graphs.emplace(gkey, exec).first;
            }
            if (capturable) GX_CUDA(cudaGraphLaunch(git->second, st));
            GX_CUDA(cudaMemcpyAsync(&mail->cs_out, d_state.ptr, sizeof cs_out, cudaMemcpyDeviceToHost, st));
            // the log holds `limit` entries; the chain writes at most up to rank_limit <= limit
            nlog = std::min<int64_t>(std::min<int64_t>(chain_k, kMailLog), limit - (rank + 1));
            GX_CUDA(cudaMemcpyAsync(mail->log, d_log.as<long long>() + rank + 1, nlog * sizeof(long long),
                                    cudaMemcpyDeviceToHost, st));
        }
        GX_CUDA(cudaEventRecord(ev_upd.b, st));
        upd_pending = true;
        // algorithmic work of the step: L read once (rank rows), the raw
        // column read, the new row written, the residual read and written
        stats.update_bytes += (double)col_bytes * (rank + 2) + 16.0 * N;
        stats.update_flops += (real ? 2.0 : 8.0) * (double)rank * N;
        fetch_red();
        if (chained) {
            cs_out = mail->cs_out;
            chain_log.assign(mail->log, mail->log + nlog);
        }
        f.pivots.push_back(pivot / n);
        f.pivots.push_back(pivot % n);
        ++rank;
        if (chained) {
            if (cs_out.stop == 4) raise(GX_EPSD, "Coulomb Cholesky residual lost positive semidefiniteness");
            for (int k = 0; k < cs_out.steps; ++k) {
                const int64_t p = chain_log[k];
                stats.update_bytes += (double)col_bytes * (rank + 2) + 16.0 * N;
                stats.update_flops += (real ? 2.0 : 8.0) * (double)rank * N;
                f.pivots.push_back(p / n);
                f.pivots.push_back(p % n);
                ++rank;
                auto e = lru_pos.find(p);  // the device consumed its cached column
                if (e != lru_pos.end()) {
                    pool.release(e->second->second);
                    lru.erase(e->second);
                    lru_pos.erase(e);
                }
                slot_of_h[p] = -1;  // already -1 on the device
                ++stats.chained_steps;
            }
            // chain length (a power of two, for few graphs): grow while chains
            // run to their end, else follow them
            int want = cs_out.active ? 2 * chain_k : cs_out.steps + 2;
            chain_k = 1;
            while (chain_k < want && chain_k < 64) chain_k *= 2;
        }
        if (red.minv < -psd) raise(GX_EPSD, "Coulomb Cholesky residual lost positive semidefiniteness");
    }
    double final_max = std::max(red.maxv, 0.0);
    if (!skipped.empty()) {
        read_diagonal(skipped, d_D.as<double>());
        GX_CUDA(gx::launch_chol_final_residual(real, d_D.as<double>(), f.L.ptr, (int)rank, N, d_res.as<double>(),
                                               st));
        GX_CUDA(gx::launch_chol_scan(d_res.as<double>(), N, d_partial.ptr, d_red.ptr, st));
        fetch_red();
        final_max = std::max(red.maxv, 0.0);
    }
    // primitive quartets of the column evaluations and their FP64 FLOP model
    // (counted per plan when launched directly, per shape when replayed)
    auto add_counts = [&](const PlanData& pd, const DeviceBuffer& counters, const std::vector<unsigned long long>* base) {
        std::vector<unsigned long long> c(2 * pd.classes.size());
        if (c.empty()) return;
        GX_CUDA(cudaMemcpyAsync(c.data(), counters.ptr, c.size() * sizeof(unsigned long long),
                                cudaMemcpyDeviceToHost, st));
        GX_CUDA(cudaStreamSynchronize(st));
        for (size_t i = 0; i < pd.classes.size(); ++i) {
            const unsigned long long v = c[2 * i] - (base ? (*base)[2 * i] : 0ull);
            stats.column_primitive_quartets += (int64_t)v;
            stats.column_model_flops += (double)v * pd.classes[i].flops_per_primitive_quartet;
        }
    };
    for (const auto& kv : plan_base) add_counts(kv.first->plan, kv.first->counters, &kv.second.second);
    for (const auto& kv : shape_base) add_counts(kv.first->plan, kv.first->counters, &kv.second.second);
    f.rank = rank;
    f.max_residual = final_max;
    stats.rank = rank;
    stats.column_pool_bytes = (double)pool.capacity * col_bytes;
    stats.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - wall0).count();
}

// Factor rows [0, rank) as complex128 into host memory.
void copy_factors(const gx_cholesky_factors& f, double* vectors) {
    if (!f.rank) return;
    cudaStream_t st = f.ctx->stream;
    const int64_t N = f.n * f.n;
    if (f.real) {
        // widened to complex128 on the device, then one copy
        DeviceBuffer wide;
        wide.reserve((size_t)f.rank * N * sizeof(double2));
        GX_CUDA(gx::launch_widen_real(f.L.as<double>(), wide.as<double2>(), f.rank * N, f.ctx->sm_count, st));
        GX_CUDA(cudaMemcpyAsync(vectors, wide.ptr, f.rank * N * sizeof(double2), cudaMemcpyDeviceToHost, st));
        GX_CUDA(cudaStreamSynchronize(st));
    } else {
        GX_CUDA(cudaMemcpyAsync(vectors, f.L.ptr, f.rank * N * sizeof(double2), cudaMemcpyDeviceToHost, st));
        GX_CUDA(cudaStreamSynchronize(st));
    }
}

}  // namespace

extern "C" int gx_cholesky(gx_context* ctx, gx_basis* b, const double* Bf, const double* Of,
                           const gx_cholesky_options* opt, double* vectors, int64_t* pivots_out, int64_t* rank_out,
                           double* max_residual) {
    return guarded([&] {
        if (!ctx || !b || !opt) raise(GX_EINVAL, "null context, basis or options");
        check_field(Bf, Of);
        *rank_out = 0;
        *max_residual = 0.0;
        std::lock_guard<std::mutex> lock(ctx->mu);
        gx_cholesky_factors f;
        try {
            cholesky_core(ctx, b, Bf, Of, opt, f);
        } catch (const ApiError&) {
            *rank_out = f.rank;
            ctx->last_cholesky = f.stats;
            throw;
        }
        ctx->last_cholesky = f.stats;
        copy_factors(f, vectors);
        std::copy(f.pivots.begin(), f.pivots.end(), pivots_out);
        *rank_out = f.rank;
        *max_residual = f.max_residual;
    });
}

extern "C" int gx_cholesky_factor(gx_context* ctx, gx_basis* b, const double* Bf, const double* Of,
                                  const gx_cholesky_options* opt, gx_cholesky_factors** out) {
    return guarded([&] {
        if (!ctx || !b || !opt || !out) raise(GX_EINVAL, "null context, basis, options or output");
        *out = nullptr;
        check_field(Bf, Of);
        std::lock_guard<std::mutex> lock(ctx->mu);
        auto f = std::make_unique<gx_cholesky_factors>();
        try {
            cholesky_core(ctx, b, Bf, Of, opt, *f);
        } catch (const ApiError&) {
            ctx->last_cholesky = f->stats;  // its rank: the rows reached when a capacity ran out
            throw;
        }
        ctx->last_cholesky = f->stats;
        *out = f.release();
    });
}

extern "C" int gx_cholesky_factors_info(const gx_cholesky_factors* f, int64_t* rank, int64_t* nao,
                                        double* max_residual, int* real) {
    return guarded([&] {
        if (!f) raise(GX_EINVAL, "null factors");
        if (rank) *rank = f->rank;
        if (nao) *nao = f->n;
        if (max_residual) *max_residual = f->max_residual;
        if (real) *real = f->real ? 1 : 0;
    });
}

extern "C" int gx_cholesky_factors_copy(const gx_cholesky_factors* f, double* vectors, int64_t* pivots) {
    return guarded([&] {
        if (!f) raise(GX_EINVAL, "null factors");
        std::lock_guard<std::mutex> lock(f->ctx->mu);
        GX_CUDA(cudaSetDevice(f->ctx->device));
        if (vectors) copy_factors(*f, vectors);
        if (pivots) std::copy(f->pivots.begin(), f->pivots.end(), pivots);
    });
}

extern "C" const void* gx_cholesky_factors_device(const gx_cholesky_factors* f) { return f ? f->L.ptr : nullptr; }

extern "C" int gx_cholesky_factors_stats(const gx_cholesky_factors* f, gx_cholesky_stats* out) {
    return guarded([&] {
        if (!f || !out) raise(GX_EINVAL, "null factors or output");
        *out = f->stats;
    });
}

extern "C" void gx_cholesky_factors_destroy(gx_cholesky_factors* f) {
    if (!f) return;
    if (f->ctx) {
        std::lock_guard<std::mutex> lock(f->ctx->mu);
        cudaSetDevice(f->ctx->device);
        f->L.release();
    }
    delete f;
}

extern "C" int gx_cholesky_last_stats(gx_context* ctx, gx_cholesky_stats* out) {
    return guarded([&] {
        if (!ctx || !out) raise(GX_EINVAL, "null context or output");
        std::lock_guard<std::mutex> lock(ctx->mu);
        *out = ctx->last_cholesky;
    });
}

// ---------------------------------------------------------------------------
// plans: build the class-sorted task list once, replay it per field
// ---------------------------------------------------------------------------

// Replay of a plan's class launches as one CUDA graph.  The graph is
// captured on the second execution with the same (stream, output, precision,
// cutoff, pair buffers, configuration) and replayed from then on; a new field
// only rewrites the pair records the graph reads.
struct PlanGraph {
    cudaGraphExec_t exec = nullptr;
    std::array<uintptr_t, 8> key{}, pending{};
    bool disabled = false;
    void reset() {
        if (exec) cudaGraphExecDestroy(exec);
        exec = nullptr;
        key = {};
        pending = {};
    }
    ~PlanGraph() { reset(); }
};

struct gx_eri_plan {
    gx_context* ctx;
    gx_basis* basis;
    PlanData data;
    int64_t total = 0;
    int last_launches = 0;
    PlanGraph graph;
    int generation = 0;  // bumped when the launch configuration changes
    int graph_replays = 0;
};

extern "C" {

int gx_context_set_stream(gx_context* ctx, void* stream) {
    return guarded([&] {
        if (!ctx) raise(GX_EINVAL, "null context");
        std::lock_guard<std::mutex> lock(ctx->mu);
        ctx->stream = stream ? static_cast<cudaStream_t>(stream) : ctx->own_stream;
    });
}

int gx_context_synchronize(gx_context* ctx) {
    return guarded([&] {
        if (!ctx) raise(GX_EINVAL, "null context");
        std::lock_guard<std::mutex> lock(ctx->mu);
        GX_CUDA(cudaSetDevice(ctx->device));
        check_status(ctx);
    });
}

int gx_eri_plan_create(gx_context* ctx, gx_basis* b, const uint32_t* quartets, int64_t nq, int64_t* offsets,
                       gx_eri_plan** out) {
    return guarded([&] {
        if (!ctx || !b) raise(GX_EINVAL, "null context or basis");
        validate_quartets(b, quartets, nq);
        std::lock_guard<std::mutex> lock(ctx->mu);
        GX_CUDA(cudaSetDevice(ctx->device));
        auto plan = std::make_unique<gx_eri_plan>();
        plan->ctx = ctx;
        plan->basis = b;
        std::vector<QuartetRequest> req((size_t)nq);
        int64_t off = 0;
        for (int64_t i = 0; i < nq; ++i) {
            const uint32_t* x = quartets + 4 * i;
            offsets[i] = off;
            req[i] = {x[0], x[1], x[2], x[3], off};
            off += b->nao_of(x[0]) * b->nao_of(x[1]) * b->nao_of(x[2]) * b->nao_of(x[3]);
        }
        offsets[nq] = off;
        plan->total = off;
        build_plan(ctx, b, req, plan->data);
        GX_CUDA(cudaStreamSynchronize(ctx->stream));
        *out = plan.release();
    });
}

int gx_eri_plan_info(const gx_eri_plan* plan, int64_t* tasks, int64_t* primitive_quartets, double* model_flops,
                     int* launches) {
    return guarded([&] {
        if (!plan) raise(GX_EINVAL, "null plan");
        if (tasks) *tasks = plan->data.ntask;
        if (primitive_quartets) *primitive_quartets = plan->data.primitive_quartets;
        if (model_flops) *model_flops = plan->data.model_flops;
        if (launches) *launches = 1 + (int)plan->data.classes.size();
    });
}

namespace {

void check_precision(int precision) {
    if (precision != GX_PRECISION_FP64 && precision != GX_PRECISION_MIXED && precision != GX_PRECISION_FP64_EXACT)
        raise(GX_EINVAL, "precision must be GX_PRECISION_FP64, GX_PRECISION_MIXED or GX_PRECISION_FP64_EXACT");
}

// Enqueue one execution of the plan, replaying its CUDA graph when the
// launch parameters repeat (see PlanGraph).
void plan_enqueue(gx_eri_plan* plan, const double* B, const double* O, int precision, double mixed_cutoff,
                  double2* out) {
    gx_context* ctx = plan->ctx;
    PlanData& pd = plan->data;
    pd.counters.reserve(std::max<size_t>(2 * pd.classes.size(), 2) * sizeof(unsigned long long));
    FieldPairs& fp = field_pairs(plan->basis, B, O);  // host work only when the field changes
    double cut = mixed_cutoff;
    uint64_t cut_bits;
    std::memcpy(&cut_bits, &cut, sizeof cut_bits);
    const std::array<uintptr_t, 8> key{(uintptr_t)ctx->stream, (uintptr_t)out, (uintptr_t)precision,
                                       (uintptr_t)cut_bits, (uintptr_t)fp.p.ptr, (uintptr_t)fp.Epool.ptr,
                                       (uintptr_t)fp.order.ptr, (uintptr_t)plan->generation};
    PlanGraph& g = plan->graph;
    const bool capturable = !g.disabled && ctx->stream != nullptr;
    if (capturable && g.exec && g.key == key) {
        GX_CUDA(cudaGraphLaunch(g.exec, ctx->stream));
        ++plan->graph_replays;
        plan->last_launches = 1 + (int)pd.classes.size();
        return;
    }
    if (capturable && g.pending == key) {
        g.reset();
        cudaGraph_t graph = nullptr;
        cudaError_t e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            try {
                plan->last_launches = execute_plan(ctx, plan->basis, B, O, pd, out, precision, mixed_cutoff,
                                                   pd.counters.as<unsigned long long>());
            } catch (...) {
                cudaStreamEndCapture(ctx->stream, &graph);
                if (graph) cudaGraphDestroy(graph);
                cudaGetLastError();
                throw;
            }
            e = cudaStreamEndCapture(ctx->stream, &graph);
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&g.exec, graph, 0);
        if (graph) cudaGraphDestroy(graph);
        if (e == cudaSuccess) {
            g.key = key;
            GX_CUDA(cudaGraphLaunch(g.exec, ctx->stream));
            ++plan->graph_replays;
            return;
        }
        // capture is not available on this stream: run eagerly from now on
        cudaGetLastError();
        g.reset();
        g.disabled = true;
    }
    plan->last_launches = execute_plan(ctx, plan->basis, B, O, pd, out, precision, mixed_cutoff,
                                       pd.counters.as<unsigned long long>());
    if (capturable) g.pending = key;
}

}  // namespace

int gx_eri_plan_execute(gx_eri_plan* plan, const double* B, const double* O, int precision, double mixed_cutoff,
                        void* out_device) {
    return guarded([&] {
        if (!plan) raise(GX_EINVAL, "null plan");
        check_field(B, O);
        check_precision(precision);
        if (!out_device) raise(GX_EINVAL, "null output pointer");
        gx_context* ctx = plan->ctx;
        std::lock_guard<std::mutex> lock(ctx->mu);
        GX_CUDA(cudaSetDevice(ctx->device));
        plan_enqueue(plan, B, O, precision, mixed_cutoff, static_cast<double2*>(out_device));
    });
}

int gx_eri_plan_class_count(const gx_eri_plan* plan) {
    if (!plan) return gx::set_error(GX_EINVAL, "null plan");
    return (int)plan->data.classes.size();
}

int gx_eri_plan_graph_replays(const gx_eri_plan* plan) {
    if (!plan) return gx::set_error(GX_EINVAL, "null plan");
    return plan->graph_replays;
}

int gx_eri_plan_profile(gx_eri_plan* plan, const double* B, const double* O, int precision, double mixed_cutoff,
                        void* out_device, gx_class_profile* out) {
    return guarded([&] {
        if (!plan || !out) raise(GX_EINVAL, "null plan or profile array");
        check_field(B, O);
        check_precision(precision);
        if (!out_device) raise(GX_EINVAL, "null output pointer");
        gx_context* ctx = plan->ctx;
        std::lock_guard<std::mutex> lock(ctx->mu);
        GX_CUDA(cudaSetDevice(ctx->device));
        PlanData& pd = plan->data;
        const size_t nc = pd.classes.size();
        pd.counters.reserve(std::max<size_t>(2 * nc, 2) * sizeof(unsigned long long));
        auto* counters = pd.counters.as<unsigned long long>();
        FieldPairs& fp = field_pairs(plan->basis, B, O);
        const gx::EriDev dev = make_dev(ctx, plan->basis, fp, static_cast<double2*>(out_device), precision,
                                        mixed_cutoff);
        cudaStream_t s = ctx->stream;
        GX_CUDA(cudaMemsetAsync(counters, 0, std::max<size_t>(2 * nc, 2) * sizeof(unsigned long long), s));
        ctx->reset_status();
        const auto& tuned = pd.tuned[precision];
        const GroupSet& gs = tuned.valid ? tuned.groups : pd.base;
        std::vector<cudaEvent_t> ev(nc + 1);
        for (auto& e : ev) GX_CUDA(cudaEventCreate(&e));
        std::vector<int> b1(nc), wpb(nc), tiles(3 * nc, 0);
        GX_CUDA(cudaEventRecord(ev[0], s));
        for (size_t ci = 0; ci < nc; ++ci) {
            launch_class(ctx, dev, pd, ci, tuned.valid ? tuned.conf[ci] : pd.defconf[ci],
                         gs.dev.as<int2>() + gs.range[ci].first, (int)gs.range[ci].second, counters, s, &b1[ci],
                         &wpb[ci], &tiles[3 * ci], gs.dev.as<int2>() + gs.lane[ci].first, (int)gs.lane[ci].second);
            GX_CUDA(cudaEventRecord(ev[ci + 1], s));
        }
        GX_CUDA(cudaEventSynchronize(ev[nc]));
        std::vector<unsigned long long> c(2 * nc);
        if (nc) GX_CUDA(cudaMemcpy(c.data(), counters, c.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
        for (size_t ci = 0; ci < nc; ++ci) {
            const PlanClass& pc = pd.classes[ci];
            gx_class_profile& o = out[ci];
            o.la = pc.key[0];
            o.lb = pc.key[1];
            o.lc = pc.key[2];
            o.ld = pc.key[3];
            o.tasks = (int64_t)pc.count;
            o.primitive_quartets = pc.primitive_quartets;
            o.fp64_quartets = (int64_t)c[2 * ci];
            o.fp32_quartets = (int64_t)c[2 * ci + 1];
            o.model_flops_per_quartet = pc.flops_per_primitive_quartet;
            float ms = 0.0f;
            GX_CUDA(cudaEventElapsedTime(&ms, ev[ci], ev[ci + 1]));
            o.ms = ms;
            const ClassConf& used = tuned.valid ? tuned.conf[ci] : pd.defconf[ci];
            o.per_group = used.per_group;
            o.warps_per_block = wpb[ci];
            o.batch = b1[ci];
            o.groups = (int64_t)gs.range[ci].second;
            o.kt = tiles[3 * ci];
            o.ct = tiles[3 * ci + 1];
            o.min_blocks = tiles[3 * ci + 2];
            o.stream = used.stream;
        }
        for (auto& e : ev) cudaEventDestroy(e);
        check_status(ctx);
    });
}

int gx_eri_plan_get_config(gx_eri_plan* plan, int precision, gx_class_config* out) {
    return guarded([&] {
        if (!plan || !out) raise(GX_EINVAL, "null plan or output");
        check_precision(precision);
        std::lock_guard<std::mutex> lock(plan->ctx->mu);
        const PlanData& pd = plan->data;
        const auto& tuned = pd.tuned[precision];
        for (size_t ci = 0; ci < pd.classes.size(); ++ci) {
            const ClassConf c = tuned.valid ? tuned.conf[ci] : pd.defconf[ci];
            out[ci] = gx_class_config{c.per_group, c.wpb, c.b1, c.kt, c.ct, c.minb, c.nostage, c.stream, c.nolane};
        }
    });
}

int gx_eri_plan_set_config(gx_eri_plan* plan, int precision, const gx_class_config* confs) {
    return guarded([&] {
        if (!plan || !confs) raise(GX_EINVAL, "null plan or configuration");
        check_precision(precision);
        gx_context* ctx = plan->ctx;
        std::lock_guard<std::mutex> lock(ctx->mu);
        GX_CUDA(cudaSetDevice(ctx->device));
        PlanData& pd = plan->data;
        std::vector<ClassConf> conf(pd.classes.size());
        for (size_t ci = 0; ci < conf.size(); ++ci) {
            const gx_class_config& c = confs[ci];
            if (c.per_group < 0 || c.warps_per_block < 0 || c.warps_per_block > 4 || c.batch < 0 || c.batch > 32 ||
                (c.kt != 0 && c.kt != 1 && c.kt != 2 && c.kt != 4) || c.ct < 0 || c.ct > 4 ||
                (c.min_blocks != 0 && c.min_blocks != 2 && c.min_blocks != 4) || (c.nostage != 0 && c.nostage != 1) ||
                (c.stream != 0 && c.stream != 1) || (c.nolane != 0 && c.nolane != 1))
                raise(GX_EINVAL, "class configuration out of range");
            conf[ci] = ClassConf{c.per_group, c.warps_per_block, c.batch, c.kt, c.ct, c.min_blocks, c.nostage,
                                 c.stream, c.nolane};
        }
        auto& tuned = pd.tuned[precision];
        make_group_set(ctx, pd, conf, tuned.groups);
        tuned.conf = conf;
        tuned.valid = true;
        GX_CUDA(cudaStreamSynchronize(ctx->stream));
        ++plan->generation;
        plan->graph.reset();
    });
}

int gx_eri_plan_autotune(gx_eri_plan* plan, const double* B, const double* O, int precision, double mixed_cutoff,
                         void* out_device, int repeats, double* default_ms, double* tuned_ms) {
    return guarded([&] {
        if (!plan) raise(GX_EINVAL, "null plan");
        check_field(B, O);
        check_precision(precision);
        if (!out_device) raise(GX_EINVAL, "null output pointer");
        if (repeats < 1 || repeats > 100) raise(GX_EINVAL, "repeats must be in [1, 100]");
        gx_context* ctx = plan->ctx;
        std::lock_guard<std::mutex> lock(ctx->mu);
        GX_CUDA(cudaSetDevice(ctx->device));
        PlanData& pd = plan->data;
        const size_t nc = pd.classes.size();
        FieldPairs& fp = field_pairs(plan->basis, B, O);
        const gx::EriDev dev = make_dev(ctx, plan->basis, fp, static_cast<double2*>(out_device), precision,
                                        mixed_cutoff);
        cudaStream_t s = ctx->stream;
        ctx->reset_status();
        cudaEvent_t e0, e1;
        GX_CUDA(cudaEventCreate(&e0));
        GX_CUDA(cudaEventCreate(&e1));
        std::vector<ClassConf> best = pd.defconf;
        double tot_default = 0.0, tot_best = 0.0;
        DeviceBuffer tmp;
        for (size_t ci = 0; ci < nc; ++ci) {
            const auto& k = pd.classes[ci].key;
            // the untuned configuration first (kept unless another is clearly
            // faster), then the previous built-in default and the sweep
            std::vector<ClassConf> cands{pd.defconf[ci]};
            if (gx::small_class(k[0], k[1], k[2], k[3])) {
                for (int per : {256, 4096}) cands.push_back(ClassConf{per, 0, 0});
            } else {
                cands.push_back(ClassConf{});
                for (int per : {16, 32, 64, 128, 256, 512, 1024})
                    for (int w : {2, 4})
                        for (int b1 : {16, 32})
                            if (!(per == 32 && w == 4 && b1 == 32)) cands.push_back(ClassConf{per, w, b1});
            }
            double best_ms = 0.0, def_ms = 0.0;
            auto time_conf = [&](const ClassConf& cf) {
                auto groups = make_groups(ctx, pd, ci, cf);
                const int ngroup = (int)groups.size();
                int nlane = 0;
                if (lane_class(pd.classes[ci])) {
                    const auto lg = make_groups(ctx, pd, ci, cf, true);
                    nlane = (int)lg.size();
                    groups.insert(groups.end(), lg.begin(), lg.end());
                }
                upload(tmp, groups, s);
                double t = 1e30;
                for (int r = 0; r <= repeats; ++r) {  // first launch warms caches
                    GX_CUDA(cudaEventRecord(e0, s));
                    launch_class(ctx, dev, pd, ci, cf, tmp.as<int2>(), ngroup, nullptr, s, nullptr, nullptr, nullptr,
                                 tmp.as<int2>() + ngroup, nlane);
                    GX_CUDA(cudaEventRecord(e1, s));
                    GX_CUDA(cudaEventSynchronize(e1));
                    float ms = 0.0f;
                    GX_CUDA(cudaEventElapsedTime(&ms, e0, e1));
                    if (r > 0) t = std::min(t, (double)ms);
                }
                return t;
            };
            for (size_t c = 0; c < cands.size(); ++c) {
                const double t = time_conf(cands[c]);
                if (c == 0) {
                    def_ms = best_ms = t;
                } else if (t < 0.97 * best_ms) {  // keep the default unless clearly faster
                    best_ms = t;
                    best[ci] = cands[c];
                }
            }
            if (!gx::small_class(k[0], k[1], k[2], k[3])) {
                // second stage: transform tiles under the chosen work split
                const int ncd = ctx->pair_class(k[2], k[3]).nab;
                for (int kt : {1, 2, 4})
                    for (int ct : {1, 2, 3, 4}) {
                        if (ncd % ct) continue;
                        ClassConf cf = best[ci];
                        cf.kt = kt;
                        cf.ct = ct;
                        const double t = time_conf(cf);
                        if (t < 0.97 * best_ms) {
                            best_ms = t;
                            best[ci] = cf;
                        }
                    }
                // third stage: the kernel variant with half the registers and
                // twice the resident warps, with and without smaller units
                {
                    ClassConf cf = best[ci];
                    cf.nostage = 1;
                    const double t = time_conf(cf);
                    if (t < 0.97 * best_ms) {
                        best_ms = t;
                        best[ci] = cf;
                    }
                }
                const ClassConf base = best[ci];
                for (int per : {0, 16, 32, 64})
                    for (int b1 : {0, 16}) {
                        ClassConf cf = base;
                        cf.minb = 4;
                        if (per) cf.per_group = per;
                        if (b1) cf.b1 = b1;
                        const double t = time_conf(cf);
                        if (t < 0.97 * best_ms) {
                            best_ms = t;
                            best[ci] = cf;
                        }
                    }
            }
            if (!gx::small_class(k[0], k[1], k[2], k[3])) {
                // fourth stage: stream mode (per-entry recurrences, small
                // shared footprint, more resident warps) on the chosen split
                const ClassConf base = best[ci];
                for (int minb : {2, 4})
                    for (int b1 : {0, 16})
                        for (int nostage : {0, 1}) {
                            ClassConf cf = base;
                            cf.stream = 1;
                            cf.minb = minb;
                            cf.b1 = b1 ? b1 : 32;
                            cf.nostage = nostage;
                            const double t = time_conf(cf);
                            if (t < 0.97 * best_ms) {
                                best_ms = t;
                                best[ci] = cf;
                            }
                        }
            }
            if (precision == GX_PRECISION_MIXED && lane_class(pd.classes[ci])) {
                // fifth stage: the FP32 entries in the generic kernel instead of the lane kernel
                ClassConf cf = best[ci];
                cf.nolane = 1;
                const double t = time_conf(cf);
                if (t < 0.97 * best_ms) {
                    best_ms = t;
                    best[ci] = cf;
                }
            }
            tot_default += def_ms;
            tot_best += best_ms;
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        check_status(ctx);
        auto& tuned = pd.tuned[precision];
        make_group_set(ctx, pd, best, tuned.groups);
        tuned.conf = best;
        tuned.valid = true;
        record_tuning(ctx, plan->basis, precision, pd, best);
        GX_CUDA(cudaStreamSynchronize(s));
        ++plan->generation;
        plan->graph.reset();
        if (default_ms) *default_ms = tot_default;
        if (tuned_ms) *tuned_ms = tot_best;
    });
}

int gx_eri_plan_counts(gx_eri_plan* plan, int64_t* fp64_quartets, int64_t* fp32_quartets, double* fp64_flops,
                       double* fp32_flops) {
    return guarded([&] {
        if (!plan) raise(GX_EINVAL, "null plan");
        std::lock_guard<std::mutex> lock(plan->ctx->mu);
        const size_t nc = plan->data.classes.size();
        std::vector<unsigned long long> c(2 * nc);
        GX_CUDA(cudaStreamSynchronize(plan->ctx->stream));
        if (nc)
            GX_CUDA(cudaMemcpy(c.data(), plan->data.counters.ptr, c.size() * sizeof(unsigned long long),
                               cudaMemcpyDeviceToHost));
        int64_t n64 = 0, n32 = 0;
        double f64 = 0.0, f32 = 0.0;
        for (size_t i = 0; i < nc; ++i) {
            n64 += (int64_t)c[2 * i];
            n32 += (int64_t)c[2 * i + 1];
            f64 += (double)c[2 * i] * plan->data.classes[i].flops_per_primitive_quartet;
            f32 += (double)c[2 * i + 1] * plan->data.classes[i].flops_per_primitive_quartet;
        }
        if (fp64_quartets) *fp64_quartets = n64;
        if (fp32_quartets) *fp32_quartets = n32;
        if (fp64_flops) *fp64_flops = f64;
        if (fp32_flops) *fp32_flops = f32;
    });
}

void gx_eri_plan_destroy(gx_eri_plan* plan) { delete plan; }

int gx_measure_fp64_peak(gx_context* ctx, double* tflops) {
    return guarded([&] {
        if (!ctx) raise(GX_EINVAL, "null context");
        std::lock_guard<std::mutex> lock(ctx->mu);
        GX_CUDA(cudaSetDevice(ctx->device));
        float ms = 0.f;
        double flops = 0.0;
        GX_CUDA(gx::run_fp64_probe(ctx->sm_count, ctx->stream, &ms, &flops));
        *tflops = flops / (ms * 1e-3) / 1e12;
    });
}

int gx_measure_fp32_peak(gx_context* ctx, double* tflops) {
    return guarded([&] {
        if (!ctx) raise(GX_EINVAL, "null context");
        std::lock_guard<std::mutex> lock(ctx->mu);
        GX_CUDA(cudaSetDevice(ctx->device));
        float ms = 0.f;
        double flops = 0.0;
        GX_CUDA(gx::run_fp32_probe(ctx->sm_count, ctx->stream, &ms, &flops));
        *tflops = flops / (ms * 1e-3) / 1e12;
    });
}

}  // extern "C"

// Canonical representatives of the finite-field orbit {(ab|cd), (cd|ab),
// (ba|dc)*, (dc|ba)*} in lexicographic order (src/eri.cpp:414-429, 825-843).
// out may be NULL to count; returns the count.
extern "C" int64_t gx_canonical_quartets(int ns, uint32_t* out) {
    int64_t n = 0;
    for (int a = 0; a < ns; ++a)
        for (int b = 0; b < ns; ++b)
            for (int c = 0; c < ns; ++c)
                for (int d = 0; d < ns; ++d) {
                    const std::array<int, 4> me{a, b, c, d};
                    if (std::array<int, 4>{c, d, a, b} < me || std::array<int, 4>{b, a, d, c} < me ||
                        std::array<int, 4>{d, c, b, a} < me)
                        continue;
                    if (out) {
                        out[4 * n] = (uint32_t)a;
                        out[4 * n + 1] = (uint32_t)b;
                        out[4 * n + 2] = (uint32_t)c;
                        out[4 * n + 3] = (uint32_t)d;
                    }
                    ++n;
                }
    return n;
}

namespace gx {
int set_error(int code, const std::string& msg) { return fail(code, msg); }
}  // namespace gx
