// Thin extern "C" shim over the reference library's own C++ API (giao::),
// compiled together with the reference's hot-path sources by
// oracle/build_ref.py.  Test infrastructure only: it lets the golden-vector
// generator and the oracle checks call the reference implementation through
// ctypes without pybind11.  Nothing in the product links it.
//
// Entry points mirror the reference bindings:
//   ref_boys               <- src/bindings.cpp:444-482 (compute_boys)
//   ref_primitive_eri      <- src/bindings.cpp:599-614 (primitive_eri)
//   ref_eri_shell          <- src/bindings.cpp:616-639 (compute_eri)
//   ref_eri_batch          <- src/bindings.cpp:672-731 (evaluate_eri_shell_quartets)
//   ref_eri_full           <- src/bindings.cpp:640-671 (compute_eri_tensor)
//   ref_schwarz            <- src/bindings.cpp:409-425 (EriSchwarzBounds)
//   ref_eri_center_derivatives <- src/derivatives.cpp:954-959
//   ref_eri_magnetic_derivatives <- src/derivatives.cpp:961-966
//   ref_eri_mixed_derivatives  <- src/derivatives.cpp:968-973
//   ref_eri_derivative_bounds  <- src/derivatives.cpp:1307-1372
//   ref_contract_eri_derivatives <- src/assembly.cpp:87-158
//   ref_cholesky_diagonal  <- src/bindings.cpp:2306-2314
//   ref_cholesky_columns   <- src/bindings.cpp:2315-2330
#include "giao_integrals/boys.hpp"
#include "assembly.hpp"
#include "giao_integrals/derivatives.hpp"
#include "giao_integrals/eri.hpp"
#include "giao_integrals/nuclear.hpp"
#include "giao_integrals/types.hpp"
#include "cholesky.hpp"

#include <complex>
#include <cstdint>
#include <cstring>
#include <exception>
#include <stdexcept>
#include <string>
#include <vector>

namespace {

thread_local std::string g_error;

int fail(const std::exception& e, int code) {
    g_error = e.what();
    return code;
}

template <typename F>
int guarded(F&& f) {
    try {
        f();
        return 0;
    } catch (const giao::BoysNumericalError& e) {
        return fail(e, -4);
    } catch (const std::invalid_argument& e) {
        return fail(e, -1);
    } catch (const std::out_of_range& e) {
        return fail(e, -2);
    } catch (const std::length_error& e) {
        return fail(e, -3);
    } catch (const std::exception& e) {
        return fail(e, -5);
    }
}

giao::Basis make_basis(int ns, const double* centers, const int* ls,
                       const int* nprims, const int* ncontrs,
                       const double* exps, const double* coefs,
                       const int* normalize) {
    std::vector<giao::Shell> shells;
    std::size_t e = 0, c = 0;
    for (int s = 0; s < ns; ++s) {
        std::vector<double> ex(exps + e, exps + e + nprims[s]);
        std::vector<double> co(coefs + c, coefs + c + (std::size_t)nprims[s] * ncontrs[s]);
        e += nprims[s];
        c += (std::size_t)nprims[s] * ncontrs[s];
        shells.emplace_back(giao::Vec3{centers[3 * s], centers[3 * s + 1], centers[3 * s + 2]},
                            (std::uint16_t)ls[s], std::move(ex), std::move(co),
                            (std::size_t)ncontrs[s],
                            normalize[s] ? giao::ContractionNormalization::normalize
                                         : giao::ContractionNormalization::as_provided);
    }
    return giao::Basis(std::move(shells));
}

giao::MagneticField make_field(const double* B, const double* O) {
    return giao::MagneticField(giao::Vec3{B[0], B[1], B[2]}, giao::Vec3{O[0], O[1], O[2]});
}

struct Packer {
    double* out;
    std::size_t pos;
};

void pack_block(const giao::ShellQuartetBlockView& block, void* user) {
    auto* p = static_cast<Packer*>(user);
    std::memcpy(p->out + 2 * p->pos, block.values.data(), block.values.size() * sizeof(giao::Complex));
    p->pos += block.values.size();
}

}  // namespace

extern "C" {

const char* ref_last_error() { return g_error.c_str(); }

int ref_boys(double zr, double zi, int nmax, int scaled, double* out, int* region,
             double* est_error, long* segments) {
    return guarded([&] {
        std::vector<giao::Complex> v((std::size_t)nmax + 1);
        auto d = giao::compute_boys({zr, zi}, v, scaled ? giao::BoysScaling::exp_z
                                                         : giao::BoysScaling::unscaled);
        std::memcpy(out, v.data(), v.size() * sizeof(giao::Complex));
        *region = (int)d.region;
        *est_error = d.estimated_absolute_error;
        *segments = (long)d.quadrature_segments;
    });
}

int ref_primitive_eri(const double* exps, const double* centers, const int* angular,
                      const double* coefs, const int* normalized, const double* B,
                      const double* O, double* out) {
    return guarded([&] {
        std::vector<giao::PrimitiveGaussian> p;
        for (int i = 0; i < 4; ++i) {
            p.emplace_back(exps[i], giao::Vec3{centers[3 * i], centers[3 * i + 1], centers[3 * i + 2]},
                           giao::CartesianExponent{(std::uint16_t)angular[3 * i],
                                                   (std::uint16_t)angular[3 * i + 1],
                                                   (std::uint16_t)angular[3 * i + 2]},
                           coefs[i], normalized[i] != 0);
        }
        auto v = giao::primitive_eri(p[0], p[1], p[2], p[3], make_field(B, O));
        out[0] = v.real();
        out[1] = v.imag();
    });
}

int ref_shell_coefficients(int ns, const double* centers, const int* ls, const int* nprims,
                           const int* ncontrs, const double* exps, const double* coefs,
                           const int* normalize, double* out) {
    return guarded([&] {
        auto basis = make_basis(ns, centers, ls, nprims, ncontrs, exps, coefs, normalize);
        std::size_t c = 0;
        for (const auto& s : basis.shells()) {
            for (double v : s.coefficients()) out[c++] = v;
        }
    });
}

int ref_eri_batch(int ns, const double* centers, const int* ls, const int* nprims,
                  const int* ncontrs, const double* exps, const double* coefs,
                  const int* normalize, const std::uint32_t* quartets, long nq,
                  const double* B, const double* O, int threads, double screening,
                  double* out, long* stats) {
    return guarded([&] {
        auto basis = make_basis(ns, centers, ls, nprims, ncontrs, exps, coefs, normalize);
        auto field = make_field(B, O);
        std::vector<giao::ShellQuartetIndex> q((std::size_t)nq);
        for (long i = 0; i < nq; ++i) {
            q[i] = {quartets[4 * i], quartets[4 * i + 1], quartets[4 * i + 2], quartets[4 * i + 3]};
        }
        std::vector<giao::EriSchwarzBounds> bounds;
        if (screening > 0.0) bounds.emplace_back(basis, field);
        Packer packer{out, 0};
        auto st = giao::evaluate_eri_shell_quartets(
            basis, q, field, {screening, (std::size_t)threads},
            bounds.empty() ? nullptr : &bounds[0], pack_block, &packer);
        stats[0] = (long)st.requested_quartets;
        stats[1] = (long)st.computed_quartets;
        stats[2] = (long)st.screened_quartets;
    });
}

int ref_eri_full(int ns, const double* centers, const int* ls, const int* nprims,
                 const int* ncontrs, const double* exps, const double* coefs,
                 const int* normalize, const double* B, const double* O, int threads,
                 double* out) {
    return guarded([&] {
        auto basis = make_basis(ns, centers, ls, nprims, ncontrs, exps, coefs, normalize);
        const std::size_t n = basis.ao_count();
        auto span = std::span<giao::Complex>(reinterpret_cast<giao::Complex*>(out), n * n * n * n);
        [[maybe_unused]] auto st =
            giao::compute_eri_tensor(basis, make_field(B, O), {0.0, (std::size_t)threads}, nullptr, span);
    });
}

int ref_nuclear_matrix(int ns, const double* centers, const int* ls, const int* nprims,
                       const int* ncontrs, const double* exps, const double* coefs,
                       const int* normalize, int nnuc, const double* charges, const double* ncenters,
                       const double* B, const double* O, double* out) {
    return guarded([&] {
        auto basis = make_basis(ns, centers, ls, nprims, ncontrs, exps, coefs, normalize);
        std::vector<giao::Nucleus> nuclei;
        for (int c = 0; c < nnuc; ++c)
            nuclei.emplace_back(charges[c], giao::Vec3{ncenters[3 * c], ncenters[3 * c + 1], ncenters[3 * c + 2]});
        const std::size_t n = basis.ao_count();
        giao::compute_nuclear_attraction_matrix(
            basis, nuclei, make_field(B, O), std::span<giao::Complex>(reinterpret_cast<giao::Complex*>(out), n * n));
    });
}

// Centre-derivative blocks (4, 3, na, nb, nc, nd) of nq quartets, packed in
// input order (compute_eri_center_derivatives, src/derivatives.cpp:954-959).
int ref_eri_center_derivatives(int ns, const double* centers, const int* ls, const int* nprims,
                               const int* ncontrs, const double* exps, const double* coefs,
                               const int* normalize, const uint32_t* quartets, long nq, const double* B,
                               const double* O, double* out) {
    return guarded([&] {
        auto basis = make_basis(ns, centers, ls, nprims, ncontrs, exps, coefs, normalize);
        const auto field = make_field(B, O);
        std::size_t off = 0;
        for (long i = 0; i < nq; ++i) {
            const auto& sh = basis.shells();
            const auto& a = sh[quartets[4 * i]];
            const auto& b = sh[quartets[4 * i + 1]];
            const auto& c = sh[quartets[4 * i + 2]];
            const auto& d = sh[quartets[4 * i + 3]];
            const std::size_t size = 12 * giao::shell_quartet_size(a, b, c, d);
            giao::compute_eri_center_derivatives(
                a, b, c, d, field, std::span<giao::Complex>(reinterpret_cast<giao::Complex*>(out) + off, size));
            off += size;
        }
    });
}

// Magnetic-derivative blocks (3, na, nb, nc, nd) of nq quartets, packed in
// input order (compute_eri_magnetic_derivatives, src/derivatives.cpp:961-966).
int ref_eri_magnetic_derivatives(int ns, const double* centers, const int* ls, const int* nprims,
                                 const int* ncontrs, const double* exps, const double* coefs,
                                 const int* normalize, const uint32_t* quartets, long nq, const double* B,
                                 const double* O, double* out) {
    return guarded([&] {
        auto basis = make_basis(ns, centers, ls, nprims, ncontrs, exps, coefs, normalize);
        const auto field = make_field(B, O);
        std::size_t off = 0;
        for (long i = 0; i < nq; ++i) {
            const auto& sh = basis.shells();
            const auto& a = sh[quartets[4 * i]];
            const auto& b = sh[quartets[4 * i + 1]];
            const auto& c = sh[quartets[4 * i + 2]];
            const auto& d = sh[quartets[4 * i + 3]];
            const std::size_t size = 3 * giao::shell_quartet_size(a, b, c, d);
            giao::compute_eri_magnetic_derivatives(
                a, b, c, d, field, std::span<giao::Complex>(reinterpret_cast<giao::Complex*>(out) + off, size));
            off += size;
        }
    });
}

// Mixed field/centre derivative blocks (4, 3, 3, na, nb, nc, nd) of nq
// quartets, packed in input order (compute_eri_mixed_derivatives,
// src/derivatives.cpp:968-973).
int ref_eri_mixed_derivatives(int ns, const double* centers, const int* ls, const int* nprims,
                              const int* ncontrs, const double* exps, const double* coefs,
                              const int* normalize, const uint32_t* quartets, long nq, const double* B,
                              const double* O, double* out) {
    return guarded([&] {
        auto basis = make_basis(ns, centers, ls, nprims, ncontrs, exps, coefs, normalize);
        const auto field = make_field(B, O);
        std::size_t off = 0;
        for (long i = 0; i < nq; ++i) {
            const auto& sh = basis.shells();
            const auto& a = sh[quartets[4 * i]];
            const auto& b = sh[quartets[4 * i + 1]];
            const auto& c = sh[quartets[4 * i + 2]];
            const auto& d = sh[quartets[4 * i + 3]];
            const std::size_t size = 36 * giao::shell_quartet_size(a, b, c, d);
            giao::compute_eri_mixed_derivatives(
                a, b, c, d, field, std::span<giao::Complex>(reinterpret_cast<giao::Complex*>(out) + off, size));
            off += size;
        }
    });
}

// Per-atom contraction of canonical centre-derivative blocks with density
// pairs and an optional complex two-particle density
// (detail::contract_eri_derivatives, src/assembly.cpp:87-158).  coulomb /
// exchange: npc / npx pairs of complex (n, n) matrices, P then Q; gamma:
// complex n^4 or null; out: complex (natom, 3), accumulated.
int ref_contract_eri_derivatives(int ns, const double* centers, const int* ls, const int* nprims,
                                 const int* ncontrs, const double* exps, const double* coefs,
                                 const int* normalize, const long* atoms, long natom, const uint32_t* quartets,
                                 long nq, const long* offsets, const double* values, int npc,
                                 const double* coulomb, int npx, const double* exchange, const double* gamma,
                                 double* out) {
    return guarded([&] {
        auto basis = make_basis(ns, centers, ls, nprims, ncontrs, exps, coefs, normalize);
        const std::size_t n = basis.ao_count();
        std::vector<std::size_t> at(atoms, atoms + ns);
        std::vector<giao::ShellQuartetIndex> q;
        for (long i = 0; i < nq; ++i)
            q.push_back({quartets[4 * i], quartets[4 * i + 1], quartets[4 * i + 2], quartets[4 * i + 3]});
        std::vector<std::size_t> off(offsets, offsets + nq + 1);
        auto cx = [](const double* p) { return reinterpret_cast<const giao::Complex*>(p); };
        std::vector<giao::detail::DensityPair> jp, kp;
        for (int i = 0; i < npc; ++i)
            jp.push_back({{cx(coulomb) + 2 * i * n * n, n * n}, {cx(coulomb) + (2 * i + 1) * n * n, n * n}});
        for (int i = 0; i < npx; ++i)
            kp.push_back({{cx(exchange) + 2 * i * n * n, n * n}, {cx(exchange) + (2 * i + 1) * n * n, n * n}});
        std::span<const giao::Complex> g;
        if (gamma) g = {cx(gamma), n * n * n * n};
        giao::detail::contract_eri_derivatives(basis, at, (std::size_t)natom, q, off,
                                               {cx(values), (std::size_t)off.back()}, jp, kp, g, {},
                                               {reinterpret_cast<giao::Complex*>(out), (std::size_t)natom * 3}, 1);
    });
}

int ref_schwarz(int ns, const double* centers, const int* ls, const int* nprims,
                const int* ncontrs, const double* exps, const double* coefs,
                const int* normalize, const double* B, const double* O, double* out) {
    return guarded([&] {
        auto basis = make_basis(ns, centers, ls, nprims, ncontrs, exps, coefs, normalize);
        giao::EriSchwarzBounds b(basis, make_field(B, O));
        std::memcpy(out, b.values().data(), b.values().size() * sizeof(double));
    });
}

// Derivative Schwarz factors per ordered shell pair
// (EriDerivativeSchwarzBounds::values, src/derivatives.cpp:1307-1372).
int ref_eri_derivative_bounds(int ns, const double* centers, const int* ls, const int* nprims,
                              const int* ncontrs, const double* exps, const double* coefs,
                              const int* normalize, const double* B, const double* O, double* out) {
    return guarded([&] {
        auto basis = make_basis(ns, centers, ls, nprims, ncontrs, exps, coefs, normalize);
        giao::EriDerivativeSchwarzBounds b(basis, make_field(B, O));
        std::memcpy(out, b.values().data(), b.values().size() * sizeof(double));
    });
}

int ref_cholesky_diagonal(int ns, const double* centers, const int* ls, const int* nprims,
                          const int* ncontrs, const double* exps, const double* coefs,
                          const int* normalize, const long* pairs, long npairs,
                          const double* B, const double* O, int threads, double* out) {
    return guarded([&] {
        auto basis = make_basis(ns, centers, ls, nprims, ncontrs, exps, coefs, normalize);
        std::vector<std::array<std::size_t, 2>> p((std::size_t)npairs);
        for (long i = 0; i < npairs; ++i) p[i] = {(std::size_t)pairs[2 * i], (std::size_t)pairs[2 * i + 1]};
        const std::size_t n = basis.ao_count();
        giao::detail::cholesky_diagonal(basis, p, make_field(B, O), std::span<double>(out, n * n),
                                        (std::size_t)threads);
    });
}

int ref_cholesky_columns(int ns, const double* centers, const int* ls, const int* nprims,
                         const int* ncontrs, const double* exps, const double* coefs,
                         const int* normalize, const long* pivots, long npiv,
                         const double* B, const double* O, int threads, double* out) {
    return guarded([&] {
        auto basis = make_basis(ns, centers, ls, nprims, ncontrs, exps, coefs, normalize);
        std::vector<std::array<std::size_t, 2>> p((std::size_t)npiv);
        for (long i = 0; i < npiv; ++i) p[i] = {(std::size_t)pivots[2 * i], (std::size_t)pivots[2 * i + 1]};
        const std::size_t n = basis.ao_count();
        auto field = make_field(B, O);
        if (B[0] == 0.0 && B[1] == 0.0 && B[2] == 0.0) {
            giao::detail::cholesky_columns(basis, p, field, std::span<double>(out, p.size() * n * n),
                                           (std::size_t)threads);
        } else {
            giao::detail::cholesky_columns(
                basis, p, field,
                std::span<giao::Complex>(reinterpret_cast<giao::Complex*>(out), p.size() * n * n),
                (std::size_t)threads);
        }
    });
}

}  // extern "C"
