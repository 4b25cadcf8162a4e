// ref_driver.cpp — runs the reference's own H|psi> and dH/dk|psi> on a
// synthetic system (test infrastructure; never part of the product path).
//
// The reference sources are compiled in the same translation unit from
// oracle/_ref/ref_all.cpp (made by oracle/refgen.py).  This driver
//   1. reads a system spec written by effmass_gb300/system.py (write_spec),
//   2. writes it as PWmat files (OUT.GKK, OUT.VR, atom.config, OUT.WG) so that
//      the reference's own readers load it (src/io/GKK.cppm:303-364,511-593;
//      src/io/RHO.cppm:143-193; src/io/ATOM.cppm:200-290; src/io/WG.cppm:237-268),
//   3. registers the synthetic pseudopotentials in an in-memory UPF registry
//      (the reference's UPF reader needs pugixml, which is absent),
//   4. calls Hamiltonian::finalize and Hamiltonian::at_k(ik)(psi, hpsi) /
//      gradient().at_k(ik)(psi, {x,y,z}) band by band
//      (src/H_psi/hamiltonian_callable.cpp:94-356,
//       src/H_psi/hamiltonian_gradient.cpp:116-294),
//   5. writes everything the reference used (lattice, G-sphere views, raw β
//      tables, λ) and its outputs to a binary fixture.
//
// Modes:
//   ref_driver golden <spec.bin> <out.bin> <workdir>
//   ref_driver density <spec.bin> <occ.txt> <out.bin> <workdir>
//   ref_driver tables <spec.bin> <out.bin> <workdir>
//   ref_driver time   <spec.bin> <workdir> <ikpt> <band0> <nbands>
//       (prints one JSON line with the seconds spent in H|psi> alone)

#include "_ref/ref_all.cpp"

#include <sys/stat.h>

namespace refdrv {

struct SpeciesSpec {
    int z = 0;
    std::vector<double> r, rab;
    int nproj = 0;
    std::vector<int> l, kbeta;
    std::vector<std::vector<double>> beta;
    std::vector<double> dion_ry;  // nproj*nproj, Rydberg
};

struct KSpec {
    int npw = 0;
    std::vector<double> K;        // npw*3, Cartesian +(k+G), bohr^-1
    std::vector<double> kinetic;  // npw, Ha
};

struct Spec {
    int n1 = 0, n2 = 0, n3 = 0;
    double A[9]{};                // bohr, rows are lattice vectors
    double ecut = 0.0;            // Ha
    int natom = 0;
    std::vector<int> atom_z;
    std::vector<double> tau;      // natom*3 fractional
    std::vector<double> vloc;     // n1*n2*n3, Ha, [i][j][k]
    std::vector<SpeciesSpec> species;
    std::vector<KSpec> kpts;
    int nband = 0;
    std::vector<std::vector<std::complex<double>>> psi;  // per k: nband*npw
};

struct Reader {
    std::FILE* f;
    template <class T> T get() {
        T v{};
        if (std::fread(&v, sizeof(T), 1, f) != 1) throw std::runtime_error("spec: truncated");
        return v;
    }
    template <class T> void arr(T* p, std::size_t n) {
        if (n && std::fread(p, sizeof(T), n, f) != n) throw std::runtime_error("spec: truncated array");
    }
};

Spec readSpec(const std::string& path) {
    Spec s;
    std::FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) throw std::runtime_error("cannot open spec " + path);
    Reader R{f};
    char magic[8];
    R.arr(magic, 8);
    if (std::memcmp(magic, "HPSISPC1", 8) != 0) throw std::runtime_error("spec: bad magic");
    s.n1 = R.get<int>(); s.n2 = R.get<int>(); s.n3 = R.get<int>();
    R.arr(s.A, 9);
    s.ecut = R.get<double>();
    s.natom = R.get<int>();
    s.atom_z.resize(s.natom);
    s.tau.resize(3 * s.natom);
    R.arr(s.atom_z.data(), s.natom);
    R.arr(s.tau.data(), 3 * s.natom);
    s.vloc.resize(static_cast<std::size_t>(s.n1) * s.n2 * s.n3);
    R.arr(s.vloc.data(), s.vloc.size());
    int nsp = R.get<int>();
    s.species.resize(nsp);
    for (auto& sp : s.species) {
        sp.z = R.get<int>();
        int nr = R.get<int>();
        sp.r.resize(nr); sp.rab.resize(nr);
        R.arr(sp.r.data(), nr); R.arr(sp.rab.data(), nr);
        sp.nproj = R.get<int>();
        sp.l.resize(sp.nproj); sp.kbeta.resize(sp.nproj); sp.beta.resize(sp.nproj);
        for (int i = 0; i < sp.nproj; ++i) {
            sp.l[i] = R.get<int>();
            sp.kbeta[i] = R.get<int>();
            sp.beta[i].resize(nr);
            R.arr(sp.beta[i].data(), nr);
        }
        sp.dion_ry.resize(static_cast<std::size_t>(sp.nproj) * sp.nproj);
        R.arr(sp.dion_ry.data(), sp.dion_ry.size());
    }
    int nk = R.get<int>();
    s.kpts.resize(nk);
    for (auto& k : s.kpts) {
        k.npw = R.get<int>();
        k.K.resize(3 * static_cast<std::size_t>(k.npw));
        k.kinetic.resize(k.npw);
        R.arr(k.K.data(), k.K.size());
        R.arr(k.kinetic.data(), k.kinetic.size());
    }
    s.nband = R.get<int>();
    s.psi.resize(nk);
    for (int ik = 0; ik < nk; ++ik) {
        s.psi[ik].resize(static_cast<std::size_t>(s.nband) * s.kpts[ik].npw);
        R.arr(reinterpret_cast<double*>(s.psi[ik].data()), 2 * s.psi[ik].size());
    }
    std::fclose(f);
    return s;
}

// ---- Fortran unformatted sequential records (4-byte length markers) ----
struct FWriter {
    std::FILE* f;
    void rec(const void* p, std::size_t nbytes) {
        int len = static_cast<int>(nbytes);
        std::fwrite(&len, 4, 1, f);
        if (nbytes) std::fwrite(p, 1, nbytes, f);
        std::fwrite(&len, 4, 1, f);
    }
};

constexpr double BOHR_A = 0.52917721067;

void alAngstrom(const Spec& s, double out[9]) {
    // The readers take AL(3,3) as 9 doubles, vector n in entries [3n, 3n+3).
    for (int i = 0; i < 9; ++i) out[i] = s.A[i] * BOHR_A;
}

int maxNpw(const Spec& s) {
    int m = 0;
    for (auto& k : s.kpts) m = std::max(m, k.npw);
    return m;
}

void writeGKK(const Spec& s, const std::string& path) {
    std::FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) throw std::runtime_error("cannot write " + path);
    FWriter W{f};
    int mg = maxNpw(s);
    int nk = static_cast<int>(s.kpts.size());
    int header[8] = {s.n1, s.n2, s.n3, mg, 1, nk, 0, 1};
    W.rec(header, sizeof header);
    W.rec(&s.ecut, sizeof(double));
    double al[9];
    alAngstrom(s, al);
    W.rec(al, sizeof al);
    std::vector<int> ngt;
    ngt.push_back(1);
    for (auto& k : s.kpts) ngt.push_back(k.npw);
    W.rec(ngt.data(), ngt.size() * sizeof(int));
    std::vector<double> buf(mg);
    for (auto& k : s.kpts) {
        std::fill(buf.begin(), buf.end(), 0.0);
        std::copy(k.kinetic.begin(), k.kinetic.end(), buf.begin());
        W.rec(buf.data(), mg * sizeof(double));
        for (int d = 0; d < 3; ++d) {
            std::fill(buf.begin(), buf.end(), 0.0);
            // PWmat stores -(k+G) (src/io/GKK.cppm:543-549)
            for (int ig = 0; ig < k.npw; ++ig) buf[ig] = -k.K[3 * ig + d];
            W.rec(buf.data(), mg * sizeof(double));
        }
    }
    std::fclose(f);
}

void writeWG(const Spec& s, const std::string& path) {
    std::FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) throw std::runtime_error("cannot write " + path);
    FWriter W{f};
    int mg = maxNpw(s);
    int nk = static_cast<int>(s.kpts.size());
    int nb = std::max(1, s.nband);
    int header[9] = {s.n1, s.n2, s.n3, nb, mg, 1, nk, 0, 1};
    W.rec(header, sizeof header);
    W.rec(&s.ecut, sizeof(double));
    double al[9];
    alAngstrom(s, al);
    W.rec(al, sizeof al);
    std::vector<int> ngt;
    ngt.push_back(1);
    for (auto& k : s.kpts) ngt.push_back(k.npw);
    W.rec(ngt.data(), ngt.size() * sizeof(int));
    std::vector<std::complex<double>> buf(mg);
    for (int ik = 0; ik < nk; ++ik) {
        for (int ib = 0; ib < nb; ++ib) {
            std::fill(buf.begin(), buf.end(), 0.0);
            if (ib < s.nband)
                for (int ig = 0; ig < s.kpts[ik].npw; ++ig)
                    buf[ig] = s.psi[ik][static_cast<std::size_t>(ib) * s.kpts[ik].npw + ig];
            W.rec(buf.data(), mg * sizeof(std::complex<double>));
        }
    }
    std::fclose(f);
}

void writeVR(const Spec& s, const std::string& path) {
    std::FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) throw std::runtime_error("cannot write " + path);
    FWriter W{f};
    int header[5] = {s.n1, s.n2, s.n3, 1, 1};
    W.rec(header, sizeof header);
    double al[9];
    alAngstrom(s, al);
    W.rec(al, sizeof al);
    W.rec(s.vloc.data(), s.vloc.size() * sizeof(double));
    std::fclose(f);
}

void writeATOM(const Spec& s, const std::string& path) {
    std::FILE* f = std::fopen(path.c_str(), "w");
    if (!f) throw std::runtime_error("cannot write " + path);
    std::fprintf(f, "%d\nLATTICE\n", s.natom);
    double al[9];
    alAngstrom(s, al);
    for (int n = 0; n < 3; ++n)
        std::fprintf(f, " %.17g %.17g %.17g\n", al[3 * n], al[3 * n + 1], al[3 * n + 2]);
    std::fprintf(f, "POSITION\n");
    for (int a = 0; a < s.natom; ++a)
        std::fprintf(f, " %d %.17g %.17g %.17g 1 1 1\n", s.atom_z[a], s.tau[3 * a], s.tau[3 * a + 1], s.tau[3 * a + 2]);
    std::fclose(f);
}

// In-memory UPF registry keyed by file basename.
std::map<std::string, const SpeciesSpec*>& registry() {
    static std::map<std::string, const SpeciesSpec*> r;
    return r;
}

struct Out {
    std::FILE* f;
    template <class T> void put(T v) { std::fwrite(&v, sizeof(T), 1, f); }
    template <class T> void arr(const T* p, std::size_t n) { if (n) std::fwrite(p, sizeof(T), n, f); }
};

std::string upfName(int z) { return std::string(ATOM::elementName(z)) + ".synthetic.UPF"; }

void setup(const Spec& s, const std::string& dir) {
    ::mkdir(dir.c_str(), 0755);
    writeGKK(s, dir + "/OUT.GKK");
    writeVR(s, dir + "/OUT.VR");
    writeATOM(s, dir + "/atom.config");
    writeWG(s, dir + "/OUT.WG");
    for (auto& sp : s.species) registry()[upfName(sp.z)] = &sp;
}

void load(Hamiltonian& H, const Spec& s, bool with_wg, bool with_d2 = false) {
    H.loadGKK("OUT.GKK");
    H.loadVR("OUT.VR");
    H.loadATOM("atom.config");
    if (with_wg) H.loadWG("OUT.WG");
    for (auto& sp : s.species) H.loadNCPP(upfName(sp.z));
    std::uint64_t feat = static_cast<std::uint64_t>(PSPFeature::Nonlocal) |
                         static_cast<std::uint64_t>(PSPFeature::DBetaq);
    if (with_d2) feat |= static_cast<std::uint64_t>(PSPFeature::D2Betaq);
    H.finalize({ExtendedCheck::NCPPAtomCoverage}, feat);
}

int golden(const std::string& spec_path, const std::string& out_path, const std::string& dir) {
    Spec s = readSpec(spec_path);
    setup(s, dir);
    Hamiltonian H(dir);
    load(H, s, true);

    std::FILE* f = std::fopen(out_path.c_str(), "wb");
    if (!f) throw std::runtime_error("cannot write " + out_path);
    Out O{f};
    O.arr("HPSIREF1", 8);
    auto A = H.gkk().meta.lattice.A();
    for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) O.put(A[i][j]);
    O.put(H.gkk().meta.lattice.volume());

    // species tables exactly as the reference interpolates them
    O.put(static_cast<int>(s.species.size()));
    for (auto& sp : s.species) {
        const auto& ncp = H.ncpp(sp.z);
        const auto& bt = H.betaqTables(sp.z);
        const auto& dbt = H.dbetaqTables(sp.z);
        O.put(sp.z);
        O.put(bt.dq_);
        O.put(bt.q_max_);
        O.put(bt.norm_coeff_);
        int nt = static_cast<int>(bt.tables_.size());
        int nq = nt ? static_cast<int>(bt.tables_[0].values.size()) : 0;
        O.put(nt);
        O.put(nq);
        for (int l = 0; l <= ncp.meta.l_max; ++l) {
            auto pb = ncp.projectorBlock(l);
            for (int ib = 0; ib < pb.B.rows; ++ib) {
                const auto& t = bt.tables_[bt.l_offset_[l] + ib];
                const auto& dt = dbt.tables_[dbt.l_offset_[l] + ib];
                O.put(l);
                O.put(ib);
                O.put(pb.B[ib, ib]);
                O.arr(t.values.data(), nq);
                O.arr(dt.values.data(), nq);
            }
        }
    }

    int nk = static_cast<int>(s.kpts.size());
    O.put(nk);
    O.put(s.nband);
    for (int ik = 0; ik < nk; ++ik) {
        auto op = H.at_k(ik);
        const auto& kv = H.gkk().currentData();
        int ng = op.dim();
        O.put(ng);
        O.arr(&kv.kPoint.x, 1); O.arr(&kv.kPoint.y, 1); O.arr(&kv.kPoint.z, 1);
        for (int ig = 0; ig < ng; ++ig) { O.put(kv.g_idx[ig].x); O.put(kv.g_idx[ig].y); O.put(kv.g_idx[ig].z); }
        for (int ig = 0; ig < ng; ++ig) { O.put(kv.Kx[ig]); O.put(kv.Ky[ig]); O.put(kv.Kz[ig]); }
        O.arr(kv.kinetic.data(), ng);
        O.arr(kv.q.data(), ng);
        O.arr(kv.theta.data(), ng);
        O.arr(kv.phi.data(), ng);
        std::vector<std::complex<double>> hpsi(ng);
        for (int ib = 0; ib < s.nband; ++ib) {
            std::span<const std::complex<double>> psi(s.psi[ik].data() + static_cast<std::size_t>(ib) * ng, ng);
            std::fill(hpsi.begin(), hpsi.end(), 0.0);
            op(psi, hpsi);
            O.arr(reinterpret_cast<const double*>(hpsi.data()), 2 * static_cast<std::size_t>(ng));
        }
        auto gop = H.gradient().at_k(ik);
        std::vector<std::complex<double>> gx(ng), gy(ng), gz(ng);
        for (int ib = 0; ib < s.nband; ++ib) {
            std::span<const std::complex<double>> psi(s.psi[ik].data() + static_cast<std::size_t>(ib) * ng, ng);
            std::fill(gx.begin(), gx.end(), 0.0);
            std::fill(gy.begin(), gy.end(), 0.0);
            std::fill(gz.begin(), gz.end(), 0.0);
            gop(psi, GradHPsi{gx, gy, gz});
            O.arr(reinterpret_cast<const double*>(gx.data()), 2 * static_cast<std::size_t>(ng));
            O.arr(reinterpret_cast<const double*>(gy.data()), 2 * static_cast<std::size_t>(ng));
            O.arr(reinterpret_cast<const double*>(gz.data()), 2 * static_cast<std::size_t>(ng));
        }
    }
    std::fclose(f);
    return 0;
}

int timeit(const std::string& spec_path, const std::string& dir, int ik, int band0, int nbands) {
    Spec s = readSpec(spec_path);
    setup(s, dir);
    Hamiltonian H(dir);
    load(H, s, false);
    auto op = H.at_k(ik);
    int ng = op.dim();
    std::vector<std::complex<double>> hpsi(ng);
    auto t0 = std::chrono::steady_clock::now();
    double checksum = 0.0;
    for (int i = 0; i < nbands; ++i) {
        int ib = (band0 + i) % s.nband;
        std::span<const std::complex<double>> psi(s.psi[ik].data() + static_cast<std::size_t>(ib) * ng, ng);
        std::fill(hpsi.begin(), hpsi.end(), 0.0);
        op(psi, hpsi);
        checksum += std::real(hpsi[0]);
    }
    auto t1 = std::chrono::steady_clock::now();
    double sec = std::chrono::duration<double>(t1 - t0).count();
    std::printf("{\"seconds\": %.9f, \"bands\": %d, \"npw\": %d, \"checksum\": %.17g}\n", sec, nbands, ng, checksum);
    return 0;
}

// Radial inputs of the beta(q) / dbeta(q)/dq tables as the reference builds
// them in Hamiltonian::finalize (src/H_psi/hamiltonian.cpp:297-316: sortByL,
// diagonalizeNonlocal, then BetaqTables / DBetaqTables from mesh r, rab and
// the rotated beta(r)), and D2BetaqTables (src/pseudo/ncpp_advance.cppm:
// 908-1085, d2 beta/dq2 for the Hessian).  Output per species: "TABREF01", z,
// mesh type (0 uniform, 1 general), nr, r[nr], rab[nr], n_proj, then per
// projector l, len and beta[len]; then the tables: nt, nq, beta_q[nt][nq],
// dbeta_q[nt][nq], d2beta_q[nt][nq] (raw, without 1/sqrt(omega)).
int tables(const std::string& spec_path, const std::string& out_path, const std::string& dir) {
    Spec s = readSpec(spec_path);
    setup(s, dir);
    Hamiltonian H(dir);
    load(H, s, true, true);
    std::FILE* f = std::fopen(out_path.c_str(), "wb");
    if (!f) throw std::runtime_error("cannot write " + out_path);
    Out O{f};
    O.arr("TABREF01", 8);
    O.put(static_cast<int>(s.species.size()));
    for (auto& sp : s.species) {
        const auto& ncp = H.ncpp(sp.z);
        O.put(sp.z);
        O.put(ncp.mesh.type == MeshType::Uniform ? 0 : 1);
        const int nr = static_cast<int>(ncp.mesh.r.size());
        O.put(nr);
        O.arr(ncp.mesh.r.data(), nr);
        O.arr(ncp.mesh.rab.data(), nr);
        const int np = static_cast<int>(ncp.nonlocal.beta.size());
        O.put(np);
        for (int i = 0; i < np; ++i) {
            O.put(ncp.nonlocal.angular_momentum[i]);
            const int len = static_cast<int>(ncp.nonlocal.beta[i].size());
            O.put(len);
            O.arr(ncp.nonlocal.beta[i].data(), len);
        }
        const auto& bt = H.betaqTables(sp.z);
        const auto& dbt = H.dbetaqTables(sp.z);
        const int nt = static_cast<int>(bt.tables_.size());
        const int nq = nt ? static_cast<int>(bt.tables_[0].values.size()) : 0;
        O.put(nt);
        O.put(nq);
        for (int t = 0; t < nt; ++t) O.arr(bt.tables_[t].values.data(), nq);
        for (int t = 0; t < nt; ++t) O.arr(dbt.tables_[t].values.data(), nq);
        const auto& d2t = H.d2betaqTables(sp.z);
        for (int t = 0; t < nt; ++t) O.arr(d2t.tables_[t].values.data(), nq);
    }
    std::fclose(f);
    return 0;
}

// Charge density through the reference's own buildDensity
// (src/support/density.cppm:41-94): the spec's k-points and bands, occupations
// read from occ_path (nkpt*nband whitespace-separated values, k-point major)
// and written as an OUT.OCC file for the reference's OCC reader
// (src/io/OCC.cppm:84-230).  Output: "RHOREF01", n1, n2, n3, rho[n1*n2*n3].
int density(const std::string& spec_path, const std::string& occ_path, const std::string& out_path,
            const std::string& dir) {
    Spec s = readSpec(spec_path);
    setup(s, dir);
    std::vector<double> occ;
    {
        std::FILE* f = std::fopen(occ_path.c_str(), "r");
        if (!f) throw std::runtime_error("cannot read " + occ_path);
        double v;
        while (std::fscanf(f, "%lf", &v) == 1) occ.push_back(v);
        std::fclose(f);
    }
    const int nk = static_cast<int>(s.kpts.size());
    if (static_cast<int>(occ.size()) != nk * s.nband) throw std::runtime_error("occupations: wrong count");
    {
        std::FILE* f = std::fopen((dir + "/OUT.OCC").c_str(), "w");
        if (!f) throw std::runtime_error("cannot write OUT.OCC");
        for (int ik = 0; ik < nk; ++ik) {
            std::fprintf(f, "KPOINTS %d: 0.0 0.0 0.0\n", ik + 1);
            for (int b = 0; b < s.nband; ++b) std::fprintf(f, "%d 0.0 %.17g\n", b + 1, occ[ik * s.nband + b]);
        }
        std::fclose(f);
    }
    GKK gkk(dir + "/OUT.GKK");
    WG wg(dir + "/OUT.WG");
    OCC oc(dir + "/OUT.OCC");
    auto rho = buildDensity(gkk, wg, oc);
    std::FILE* f = std::fopen(out_path.c_str(), "wb");
    if (!f) throw std::runtime_error("cannot write " + out_path);
    Out O{f};
    O.arr("RHOREF01", 8);
    O.put(s.n1);
    O.put(s.n2);
    O.put(s.n3);
    O.arr(rho.data(), rho.size());
    std::fclose(f);
    return 0;
}

}  // namespace refdrv

// UPF from the in-memory registry (replaces the pugixml reader of
// src/pseudo/io/upf.cppm:182-213 for synthetic pseudopotentials).
UPF::UPF(const std::string& filename) : filename_(filename) {
    auto base = std::filesystem::path(filename).filename().string();
    auto it = refdrv::registry().find(base);
    if (it == refdrv::registry().end()) throw std::runtime_error("UPF registry: no entry for " + base);
    const auto& sp = *it->second;
    int nr = static_cast<int>(sp.r.size());
    header_.element = std::string(ATOM::elementName(sp.z));
    header_.pseudo_type = "NC";
    header_.relativistic = "scalar";
    header_.z_valence = 4.0;
    int lmax = 0;
    for (int l : sp.l) lmax = std::max(lmax, l);
    header_.l_max = lmax;
    header_.mesh_size = nr;
    header_.number_of_wfc = 0;
    header_.number_of_proj = sp.nproj;
    mesh_.r = sp.r;
    mesh_.rab = sp.rab;
    vloc_.assign(nr, 0.0);
    rho_at_.assign(nr, 0.0);
    nonlocal_.beta = sp.beta;
    nonlocal_.lll = sp.l;
    nonlocal_.kbeta = sp.kbeta;
    nonlocal_.rcut.assign(sp.nproj, sp.r.back());
    nonlocal_.dion.rows = sp.nproj;
    nonlocal_.dion.cols = sp.nproj;
    nonlocal_.dion.data = sp.dion_ry;
}

int main(int argc, char** argv) {
    try {
        std::string mode = argc > 1 ? argv[1] : "";
        if (mode == "golden" && argc == 5) return refdrv::golden(argv[2], argv[3], argv[4]);
        if (mode == "tables" && argc == 5) return refdrv::tables(argv[2], argv[3], argv[4]);
        if (mode == "density" && argc == 6) return refdrv::density(argv[2], argv[3], argv[4], argv[5]);
        if (mode == "time" && argc == 7)
            return refdrv::timeit(argv[2], argv[3], std::atoi(argv[4]), std::atoi(argv[5]), std::atoi(argv[6]));
        std::fprintf(stderr, "usage: ref_driver golden <spec> <out> <dir> | density <spec> <occ> <out> <dir> | "
                             "time <spec> <dir> <ik> <b0> <nb>\n");
        return 2;
    } catch (const std::exception& e) {
        std::fprintf(stderr, "ref_driver: %s\n", e.what());
        return 1;
    }
}
