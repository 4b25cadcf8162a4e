// hpsi_gb300.hpp — header-only C++20 mirror of the reference's H_psi operator
// API (src/H_psi/hamiltonian.cppm:115-310) over the C ABI of hpsi_gb300.h.
//
//   hpsi::Hamiltonian H(system);               // Hamiltonian::finalize
//   auto op = H.at_k(ik, kpoint);               // Hamiltonian::at_k
//   op(psi, hpsi);                              // Callable::operator()(psi, hpsi)
//   op(n_bands, psi, hpsi);                     // Callable::operator()(n_bands, psi, hpsi)
//   op.dim(); op.set_ikpt(j);                   // Callable::dim / set_ikpt
//   H.gradient().at_k(ik)(psi, {dx, dy, dz});   // Gradient::Callable::operator()
//
// Errors become the exception types the reference throws: HPSI_ERR_BAD_ARG ->
// std::invalid_argument, HPSI_ERR_RANGE -> std::domain_error, HPSI_ERR_STATE ->
// std::runtime_error, others -> std::runtime_error.  Spans of host memory are
// copied in and out inside each call; with device spans (set `on_device`)
// the work is queued on `stream`.
#pragma once

#include <complex>
#include <span>
#include <stdexcept>
#include <string>

#include "hpsi_gb300.h"

namespace hpsi {

inline void check(int status, const hpsi_ctx* ctx)
{
    if (status == HPSI_OK) return;
    std::string msg = hpsi_last_error(ctx);
    switch (status) {
        case HPSI_ERR_BAD_ARG: throw std::invalid_argument(msg);
        case HPSI_ERR_RANGE: throw std::domain_error(msg);
        default: throw std::runtime_error(msg);
    }
}

// Outputs of dH/dk_{x,y,z}|psi>; an empty span skips that direction
// (the reference's GradHPsi, src/H_psi/hamiltonian.cppm:66-70).
struct GradHPsi {
    std::span<std::complex<double>> x;
    std::span<std::complex<double>> y;
    std::span<std::complex<double>> z;
};

class Hamiltonian;
// plane-wave count of a bound k-point slot (Callable::dim); std::runtime_error
// for an unbound slot (hpsi_dim records no message, so it is written here)
inline int slot_dim(const Hamiltonian* H, int ikpt);

class Hamiltonian {
public:
    explicit Hamiltonian(const hpsi_system& sys, int precision = HPSI_PREC_FP64)
        : precision_(precision)
    {
        check(hpsi_ctx_create(&sys, &ctx_), nullptr);
    }
    ~Hamiltonian() { if (ctx_) hpsi_ctx_destroy(ctx_); }
    Hamiltonian(const Hamiltonian&) = delete;
    Hamiltonian& operator=(const Hamiltonian&) = delete;

    hpsi_ctx* ctx() const { return ctx_; }
    int precision() const { return precision_; }

    void set_kpoint(int ikpt, const hpsi_kpoint& kp) { check(hpsi_set_kpoint(ctx_, ikpt, &kp), ctx_); }

    class Callable {
    public:
        Callable() = default;

        // hpsi += H psi (one band)
        void operator()(std::span<const std::complex<double>> psi, std::span<std::complex<double>> hpsi) const
        {
            (*this)(1, psi, hpsi);
        }

        // hpsi[b] += H psi[b], band-major blocks of dim() values
        void operator()(int n_bands, std::span<const std::complex<double>> psi,
                        std::span<std::complex<double>> hpsi) const
        {
            const size_t need = static_cast<size_t>(n_bands) * static_cast<size_t>(dim());
            if (n_bands < 0 || psi.size() < need || hpsi.size() < need)
                throw std::invalid_argument("H|psi>: spans shorter than n_bands * dim()");
            check(hpsi_apply(parent_->ctx_, ikpt_, n_bands, reinterpret_cast<const double*>(psi.data()),
                             reinterpret_cast<double*>(hpsi.data()), flags(), stream_),
                  parent_->ctx_);
        }

        int dim() const { return slot_dim(parent_, ikpt_); }

        // Rebind to another (already set) k-point slot; on an unbound slot
        // this throws std::runtime_error and the Callable keeps its slot.
        void set_ikpt(int ikpt)
        {
            (void)slot_dim(parent_, ikpt);
            ikpt_ = ikpt;
        }

        // Device-resident spans, queued on `stream` (cudaStream_t).
        void on_device(void* stream) { device_ = true; stream_ = stream; }

    private:
        friend class Hamiltonian;
        Callable(const Hamiltonian* parent, int ikpt) : parent_(parent), ikpt_(ikpt) { (void)dim(); }
        int flags() const { return parent_->precision_ | (device_ ? HPSI_DEVICE_PTRS : 0); }
        const Hamiltonian* parent_ = nullptr;
        int ikpt_ = 0;
        bool device_ = false;
        void* stream_ = nullptr;
    };

    Callable at_k(int ikpt) const { return Callable(this, ikpt); }
    Callable at_k(int ikpt, const hpsi_kpoint& kp)
    {
        set_kpoint(ikpt, kp);
        return Callable(this, ikpt);
    }

    class Gradient {
    public:
        class Callable {
        public:
            Callable() = default;
            // out.{x,y,z}[b] += dH/dk_alpha psi[b]; empty spans are skipped
            void operator()(std::span<const std::complex<double>> psi, GradHPsi out, int n_bands = 1) const
            {
                const int npw = dim();
                const size_t need = static_cast<size_t>(n_bands) * static_cast<size_t>(npw);
                auto ptr = [&](std::span<std::complex<double>> s) -> double* {
                    if (s.empty()) return nullptr;
                    if (s.size() < need) throw std::invalid_argument("dH/dk: output span too short");
                    return reinterpret_cast<double*>(s.data());
                };
                if (psi.size() < need) throw std::invalid_argument("dH/dk: psi span too short");
                check(hpsi_grad_apply(parent_->ctx_, ikpt_, n_bands, reinterpret_cast<const double*>(psi.data()),
                                      ptr(out.x), ptr(out.y), ptr(out.z), parent_->precision_, nullptr),
                      parent_->ctx_);
            }
            int dim() const { return slot_dim(parent_, ikpt_); }

        private:
            friend class Gradient;
            Callable(const Hamiltonian* parent, int ikpt) : parent_(parent), ikpt_(ikpt) { (void)dim(); }
            const Hamiltonian* parent_ = nullptr;
            int ikpt_ = 0;
        };
        Callable at_k(int ikpt) const { return Callable(parent_, ikpt); }

    private:
        friend class Hamiltonian;
        explicit Gradient(const Hamiltonian* parent) : parent_(parent) {}
        const Hamiltonian* parent_;
    };
    Gradient gradient() const { return Gradient(this); }

private:
    hpsi_ctx* ctx_ = nullptr;
    int precision_ = HPSI_PREC_FP64;
};

inline int slot_dim(const Hamiltonian* H, int ikpt)
{
    const int n = hpsi_dim(H->ctx(), ikpt);
    if (n == HPSI_ERR_STATE) throw std::runtime_error("k-point slot " + std::to_string(ikpt) + " is not bound");
    if (n < 0) check(n, H->ctx());
    return n;
}

}  // namespace hpsi
