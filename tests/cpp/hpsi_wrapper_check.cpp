// hpsi_wrapper_check.cpp — drives the header-only C++ mirror of the
// reference's operator API (include/hpsi_gb300.hpp) against a golden record
// of the reference's own H|psi> and dH/dk|psi>, linked to libhpsi_gb300.so.
//
//   hpsi_wrapper_check <case.bin>
//
// The case file (written by tests/test_gpu_cpp_wrapper.py) holds a system, one
// k-point, nb bands of psi and the reference's hpsi and grad.  Checks, each
// printed on one line; the exit status is the number of failures:
//   * Callable::operator()(n_bands, psi, hpsi) and the one-band form, which
//     accumulate (hpsi += H psi), within 1e-12 of the reference;
//   * Gradient::Callable with all three directions, and with an empty span
//     (that direction skipped, the others unchanged);
//   * set_ikpt to another bound slot, and to an unbound one (runtime_error,
//     the Callable keeps its slot);
//   * device spans queued on a stream (on_device);
//   * exception mapping: spans shorter than n_bands * dim() throw
//     std::invalid_argument, q beyond the beta table's q_max throws
//     std::domain_error (the reference's BetaqTables::interpolate).
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "hpsi_gb300.hpp"

using cd = std::complex<double>;

namespace {

struct Reader {
    std::FILE* f;
    template <class T> T get()
    {
        T v{};
        if (std::fread(&v, sizeof(T), 1, f) != 1) throw std::runtime_error("case file truncated");
        return v;
    }
    template <class T> std::vector<T> arr(size_t n)
    {
        std::vector<T> v(n);
        if (n && std::fread(v.data(), sizeof(T), n, f) != n) throw std::runtime_error("case file truncated");
        return v;
    }
};

double rel_err(const std::vector<cd>& a, const std::vector<cd>& b)
{
    double num = 0, den = 0;
    for (size_t i = 0; i < a.size(); ++i) {
        num += std::norm(a[i] - b[i]);
        den += std::norm(b[i]);
    }
    return std::sqrt(num / (den > 0 ? den : 1e-300));
}

int failures = 0;
void report(bool ok, const std::string& what)
{
    std::printf("%s %s\n", ok ? "ok  " : "FAIL", what.c_str());
    if (!ok) ++failures;
}

}  // namespace

int main(int argc, char** argv)
{
    if (argc != 2) {
        std::fprintf(stderr, "usage: %s case.bin\n", argv[0]);
        return 99;
    }
    std::FILE* f = std::fopen(argv[1], "rb");
    if (!f) return 98;
    Reader R{f};
    // system
    hpsi_system sys{};
    sys.n1 = R.get<int>(); sys.n2 = R.get<int>(); sys.n3 = R.get<int>();
    auto lat = R.arr<double>(9);
    for (int i = 0; i < 9; ++i) sys.lattice[i] = lat[i];
    sys.omega = R.get<double>();
    const int natom = R.get<int>();
    auto atom_species = R.arr<int>(natom);
    auto tau = R.arr<double>(3 * (size_t)natom);
    const int np = R.get<int>();
    auto proj_l = R.arr<int>(np);
    auto lam = R.arr<double>(np);
    const int nq = R.get<int>();
    const double dq = R.get<double>(), q_max = R.get<double>();
    auto beta_q = R.arr<double>((size_t)np * nq);
    auto dbeta_q = R.arr<double>((size_t)np * nq);
    auto v_loc = R.arr<double>((size_t)sys.n1 * sys.n2 * sys.n3);
    hpsi_species sp{np, proj_l.data(), lam.data(), nq, dq, q_max, beta_q.data(), dbeta_q.data()};
    sys.v_loc = v_loc.data();
    sys.n_species = 1;
    sys.species = &sp;
    sys.n_atoms = natom;
    sys.atom_species = atom_species.data();
    sys.atom_tau = tau.data();
    // k-point and bands
    const int npw = R.get<int>();
    auto kf = R.arr<double>(3);
    auto g_idx = R.arr<int>(3 * (size_t)npw);
    auto kvec = R.arr<double>(3 * (size_t)npw);
    auto kin = R.arr<double>((size_t)npw);
    hpsi_kpoint kp{npw, {kf[0], kf[1], kf[2]}, g_idx.data(), kvec.data(), kin.data()};
    const int nb = R.get<int>();
    auto psi = R.arr<cd>((size_t)nb * npw);
    auto href = R.arr<cd>((size_t)nb * npw);
    std::vector<std::vector<cd>> gref(3);
    for (auto& g : gref) g = R.arr<cd>((size_t)nb * npw);
    std::fclose(f);

    const size_t nel = (size_t)nb * npw;
    try {
        hpsi::Hamiltonian H(sys);  // FP64: the parity path
        auto op = H.at_k(0, kp);
        report(op.dim() == npw, "dim() == npw");
        std::vector<cd> out(nel, cd(0, 0));
        op(nb, psi, out);
        const double e = rel_err(out, href);
        report(e <= 1e-12, "Callable(n_bands, psi, hpsi) rel err " + std::to_string(e));
        // one band, accumulating into a non-zero hpsi
        std::vector<cd> one((size_t)npw, cd(0.25, -0.5)), ref1((size_t)npw);
        for (int g = 0; g < npw; ++g) ref1[g] = cd(0.25, -0.5) + href[(size_t)(nb - 1) * npw + g];
        op(std::span<const cd>(psi.data() + (size_t)(nb - 1) * npw, npw), one);
        report(rel_err(one, ref1) <= 1e-12, "Callable(psi, hpsi) accumulates");
        // gradient, all directions, then y skipped
        std::vector<cd> gx(nel), gy(nel), gz(nel);
        H.gradient().at_k(0)(psi, hpsi::GradHPsi{gx, gy, gz}, nb);
        const double eg = std::max({rel_err(gx, gref[0]), rel_err(gy, gref[1]), rel_err(gz, gref[2])});
        report(eg <= 1e-12, "Gradient::Callable rel err " + std::to_string(eg));
        std::vector<cd> hx(nel), hz(nel);
        H.gradient().at_k(0)(psi, hpsi::GradHPsi{hx, {}, hz}, nb);
        report(rel_err(hx, gref[0]) <= 1e-12 && rel_err(hz, gref[2]) <= 1e-12, "empty GradHPsi span skips y");
        // set_ikpt: slot 3 bound to the same k-point, then an unbound slot
        H.set_kpoint(3, kp);
        op.set_ikpt(3);
        std::vector<cd> out3(nel);
        op(nb, psi, out3);
        report(rel_err(out3, href) <= 1e-12, "set_ikpt(3) rebinds");
        bool threw = false;
        try { op.set_ikpt(7); } catch (const std::runtime_error&) { threw = true; }
        report(threw, "set_ikpt(unbound) throws std::runtime_error");
        std::vector<cd> out4(nel);
        op(nb, psi, out4);  // still bound to slot 3
        report(rel_err(out4, href) <= 1e-12, "a failed set_ikpt keeps the slot");
        // device spans on a stream
        cd *dp = nullptr, *dh = nullptr;
        cudaStream_t st = nullptr;
        bool dev_ok = cudaMalloc(&dp, nel * sizeof(cd)) == cudaSuccess && cudaMalloc(&dh, nel * sizeof(cd)) == cudaSuccess &&
                      cudaStreamCreate(&st) == cudaSuccess;
        if (dev_ok) {
            cudaMemcpy(dp, psi.data(), nel * sizeof(cd), cudaMemcpyHostToDevice);
            cudaMemset(dh, 0, nel * sizeof(cd));
            auto dop = H.at_k(0);
            dop.on_device(st);
            dop(nb, std::span<const cd>(dp, nel), std::span<cd>(dh, nel));
            cudaStreamSynchronize(st);
            std::vector<cd> back(nel);
            cudaMemcpy(back.data(), dh, nel * sizeof(cd), cudaMemcpyDeviceToHost);
            report(rel_err(back, href) <= 1e-12, "device spans on a stream");
        } else {
            report(false, "device buffers");
        }
        if (dp) cudaFree(dp);
        if (dh) cudaFree(dh);
        if (st) cudaStreamDestroy(st);
        // exception mapping
        threw = false;
        try { op(nb, std::span<const cd>(psi.data(), nel - 1), out); } catch (const std::invalid_argument&) { threw = true; }
        report(threw, "short span throws std::invalid_argument");
        hpsi_species sp2 = sp;
        double qtop = 0;
        for (int g = 0; g < npw; ++g) qtop = std::max(qtop, std::sqrt(2.0 * kin[g]));
        sp2.q_max = 0.5 * qtop;
        hpsi_system sys2 = sys;
        sys2.species = &sp2;
        hpsi::Hamiltonian H2(sys2);
        threw = false;
        try { H2.set_kpoint(0, kp); } catch (const std::domain_error&) { threw = true; }
        report(threw, "q > q_max throws std::domain_error");
    } catch (const std::exception& ex) {
        std::printf("FAIL unexpected exception: %s\n", ex.what());
        ++failures;
    }
    return failures;
}
