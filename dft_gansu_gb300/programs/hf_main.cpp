// HF_main in C++ over the C ABI of libgansu_gb300 (include/gansu_gb300.h): the
// compiled counterpart of the reference's HF_main (src/HF_main.cu:40-62):
//
//     HF_main -x water.xyz -g sto-3g -m rhf [--key value ...] [-p recipe.txt]
//
// Parameters are parsed as gansu::ParameterManager parses them
// (src/parameter_manager.cpp:40-224): the same keys and defaults, the short
// options -m -v -p -x -g -ag -c, `--key value` pairs, values lower-cased except
// file names, unknown keys rejected, and a `-p` recipe (`key = value` lines,
// `#` comments) filling the keys the command line did not set.  The method
// (rhf / uhf / rohf) is solved on the GPU, the report follows RHF::report /
// HF::report (src/rhf.cu:335-360, src/hf.cu:403-430: molecule and basis
// summary, Mulliken charges, calculation summary with the total energy and the
// computing time), and the orbitals go to output.molden in the working
// directory (export_molden_file, src/rhf.cu:363-425).  initial_guess = sad
// superposes atomic densities from RHF (even Z) or ROHF doublet (odd Z) solves
// of the isolated atoms, as the reference's SAD generator makes them.
//
// A basis given by name (`-g cc-pvdz`) is looked up in the basis/ directory
// next to this program when no file of that name exists.  Errors end the
// program with status 1 (engine errors, with the engine's message) or 2
// (invalid command line).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <map>
#include <set>
#include <sstream>
#include <stdexcept>
#include <string>
#include <unistd.h>
#include <vector>

#include "gansu_gb300.h"

namespace {

// ------------------------------------------------------------ parameters
const std::vector<std::pair<std::string, std::string>>& defaults()
{
    static const std::vector<std::pair<std::string, std::string>> d = {
        {"parameter_file", ""}, {"xyzfilename", ""}, {"gbsfilename", ""}, {"verbose", "0"}, {"method", "rhf"},
        {"charge", "0"}, {"beta_to_alpha", "0"}, {"eri_method", "stored"}, {"auxiliary_gbsfilename", ""},
        {"maxiter", "100"}, {"convergence_energy_threshold", "1e-6"}, {"schwarz_screening_threshold", "1e-12"},
        {"initial_guess", "core"}, {"convergence_method", "diis"}, {"damping_factor", "0.9"}, {"diis_size", "8"},
        {"diis_include_transform", "0"}, {"rohf_parameter_name", "roothaan"}, {"geometry_optimization", "0"},
        {"geometry_optimization_method", "powell"}, {"export_sad_cache", "0"},
        // keys of this engine, same parsing rules
        {"precision", "fp64"}, {"mixed_threshold", "1e-7"}, {"incremental_fock", "0"}, {"spherical", "0"},
        {"eigensolver", "syevd"}};
    return d;
}

class ParameterManager {
public:
    ParameterManager()
    {
        for (const auto& kv : defaults()) v_[kv.first] = kv.second;
    }
    void set(const std::string& key, const std::string& value)
    {
        if (!v_.count(key)) throw std::invalid_argument("Unknown parameter: " + key);
        static const std::set<std::string> keep = {"xyzfilename", "gbsfilename", "parameter_file",
                                                   "auxiliary_gbsfilename"};
        std::string s = value;
        if (!keep.count(key)) std::transform(s.begin(), s.end(), s.begin(), ::tolower);
        v_[key] = s;
    }
    static std::string default_of(const std::string& key)
    {
        for (const auto& kv : defaults())
            if (kv.first == key) return kv.second;
        return std::string();
    }
    const std::string& str(const std::string& key) const { return v_.at(key); }
    int integer(const std::string& key) const { return std::stoi(v_.at(key)); }
    double real(const std::string& key) const { return std::stod(v_.at(key)); }
    bool flag(const std::string& key) const
    {
        const std::string& s = v_.at(key);
        return !(s.empty() || s == "0" || s == "false");
    }
    void parse_command_line(int argc, char** argv, int first)
    {
        static const std::map<std::string, std::string> shorts = {
            {"-m", "method"}, {"-v", "verbose"}, {"-p", "parameter_file"}, {"-x", "xyzfilename"},
            {"-g", "gbsfilename"}, {"-ag", "auxiliary_gbsfilename"}, {"-c", "charge"}};
        for (int i = first; i < argc; i += 2) {
            const std::string k = argv[i];
            std::string key;
            if (shorts.count(k)) key = shorts.at(k);
            else if (k.rfind("--", 0) == 0) key = k.substr(2);
            if (key.empty() || i + 1 >= argc) throw std::invalid_argument("Invalid option: " + k);
            set(key, argv[i + 1]);
        }
        if (!v_["parameter_file"].empty()) load_recipe(v_["parameter_file"]);
    }
    // `key = value` lines; keys given on the command line keep their values
    void load_recipe(const std::string& path)
    {
        std::ifstream in(path);
        if (!in) throw std::runtime_error("cannot open parameter file " + path);
        std::string line;
        while (std::getline(in, line)) {
            line = line.substr(0, line.find('#'));
            const size_t eq = line.find('=');
            if (eq == std::string::npos) continue;
            const std::string k = trim(line.substr(0, eq)), val = trim(line.substr(eq + 1));
            if (k.empty()) continue;
            if (!v_.count(k)) throw std::invalid_argument("Unknown parameter: " + k);
            if (v_[k] == default_of(k)) set(k, val);  // a value the command line changed is kept
        }
    }

private:
    static std::string trim(const std::string& s)
    {
        const size_t a = s.find_first_not_of(" \t\r\n"), b = s.find_last_not_of(" \t\r\n");
        return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
    }
    std::map<std::string, std::string> v_;
};

// ------------------------------------------------------------ helpers
struct EngineError : std::runtime_error {
    using std::runtime_error::runtime_error;
};

void check(int st, const char* what)
{
    if (st != HF_OK) throw EngineError(std::string(what) + ": " + hf_last_error());
}

void cuda_check(cudaError_t e, const char* what)
{
    if (e != cudaSuccess) throw EngineError(std::string(what) + ": " + cudaGetErrorString(e));
}

const char* kSymbols[] = {"H",  "He", "Li", "Be", "B",  "C",  "N",  "O",  "F",  "Ne", "Na", "Mg", "Al", "Si",
                          "P",  "S",  "Cl", "Ar", "K",  "Ca", "Sc", "Ti", "V",  "Cr", "Mn", "Fe", "Co", "Ni",
                          "Cu", "Zn", "Ga", "Ge", "As", "Se", "Br", "Kr"};

std::string symbol(int z) { return (z >= 1 && z <= 36) ? kSymbols[z - 1] : "X"; }

std::string program_dir(const char* argv0)
{
    char buf[4096];
    const ssize_t n = readlink("/proc/self/exe", buf, sizeof(buf) - 1);
    std::string p = n > 0 ? std::string(buf, static_cast<size_t>(n)) : std::string(argv0);
    const size_t s = p.rfind('/');
    return s == std::string::npos ? std::string(".") : p.substr(0, s);
}

bool exists(const std::string& p) { return std::ifstream(p).good(); }

// a file as given, else the bundled basis of that name
std::string basis_path(const std::string& name, const std::string& dir)
{
    if (exists(name)) return name;
    std::string f = name;
    if (f.size() < 4 || f.substr(f.size() - 4) != ".gbs") f += ".gbs";
    const std::string cand = dir + "/basis/" + f;
    if (!exists(cand)) throw std::runtime_error("basis set '" + name + "' not found (nor " + cand + ")");
    return cand;
}

// device buffer of doubles, released at scope end
struct DevBuf {
    double* p = nullptr;
    explicit DevBuf(size_t n) { cuda_check(cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(double)), "cudaMalloc"); }
    ~DevBuf() { cudaFree(p); }
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    std::vector<double> host(size_t n) const
    {
        std::vector<double> h(n);
        cuda_check(cudaMemcpy(h.data(), p, n * sizeof(double), cudaMemcpyDeviceToHost), "cudaMemcpy");
        return h;
    }
};

struct Molecule {
    hf_molecule* h = nullptr;
    int nbf = 0, nprim = 0, natom = 0, nel = 0, na = 0, nb = 0;
    std::vector<hf_primitive_shell> prims;
    std::vector<double> cgto;
    std::vector<hf_atom> atoms;
    ~Molecule() { hf_molecule_destroy(h); }
    void fill()
    {
        check(hf_molecule_sizes(h, &nbf, &nprim, &natom, &nel, &na, &nb), "hf_molecule_sizes");
        prims.resize(nprim);
        cgto.resize(nbf);
        atoms.resize(natom);
        check(hf_molecule_get(h, prims.data(), cgto.data(), atoms.data()), "hf_molecule_get");
    }
    // (first basis function, count) of every atom
    std::vector<std::pair<int, int>> atom_ranges() const
    {
        std::vector<std::pair<int, int>> r(natom, {1 << 30, 0});
        std::vector<int> hi(natom, 0);
        for (const auto& p : prims) {
            const int a = p.atom_index, lo = static_cast<int>(p.basis_index);
            const int nc = (p.shell_type + 1) * (p.shell_type + 2) / 2;
            r[a].first = std::min(r[a].first, lo);
            hi[a] = std::max(hi[a], lo + nc);
        }
        for (int a = 0; a < natom; ++a) r[a].second = hi[a] - r[a].first;
        return r;
    }
};

struct Engine {
    hf_engine* h = nullptr;
    ~Engine() { hf_engine_destroy(h); }
};

const std::map<std::string, std::vector<double>>& rohf_couplings()
{
    // (A_cc, B_cc, A_oo, B_oo, A_vv, B_vv) by rohf_parameter_name (src/rohf.cu:30-39)
    static const std::map<std::string, std::vector<double>> c = {
        {"roothaan", {-0.5, 1.5, 0.5, 0.5, 1.5, -0.5}},
        {"mcweeny-diercksen", {1.0 / 3, 2.0 / 3, 1.0 / 3, 1.0 / 3, 2.0 / 3, 1.0 / 3}},
        {"davidson", {0.5, 1.0, 0.0, 1.0, 1.0, 0.0}},
        {"guest-saunders", {0.5, 0.5, 0.5, 0.5, 0.5, 0.5}},
        {"binkley-pople-dobosh", {0.5, 0.5, 1.0, 0.0, 0.0, 1.0}},
        {"faegri-manne", {0.5, 0.5, 1.0, 0.0, 0.5, 0.5}},
        {"goddard", {0.5, 0.5, 0.5, 0.0, 1.0, 0.0}},
        {"plakhutin-gorelik-breslavskaya", {0.0, 1.0, 1.0, 0.0, 1.0, 0.0}}};
    return c;
}

// alpha and beta densities of the isolated atom z (RHF for even Z, ROHF doublet for odd Z)
void atomic_density(int z, const std::string& gbs, std::vector<double>& da, std::vector<double>& db)
{
    static std::map<int, std::pair<std::vector<double>, std::vector<double>>> cache;
    auto it = cache.find(z);
    if (it == cache.end()) {
        hf_atom atom{z, 0.0, 0.0, 0.0};
        Molecule m;
        check(hf_molecule_from_atoms(&atom, 1, gbs.c_str(), 0, 0, &m.h), "hf_molecule_from_atoms");
        m.fill();
        Engine e;
        check(hf_engine_create(m.prims.data(), m.nprim, m.cgto.data(), m.nbf, m.atoms.data(), 1, 1e-12, &e.h),
              "hf_engine_create");
        hf_scf_options o;
        hf_scf_options_default(&o);
        o.convergence_threshold = 1e-10;
        o.max_iter = 300;
        hf_scf_result r;
        const size_t nn = static_cast<size_t>(m.nbf) * m.nbf;
        DevBuf a(nn), b(nn);
        std::vector<double> ha, hb;
        if (z % 2 == 0) {
            check(hf_rhf_scf(e.h, z, &o, &r, a.p, nullptr, nullptr, nullptr), "SAD atomic RHF");
            ha = a.host(nn);
            for (auto& x : ha) x *= 0.5;
            hb = ha;
        } else {
            check(hf_rohf_scf(e.h, (z + 1) / 2, (z - 1) / 2, rohf_couplings().at("roothaan").data(), &o, &r, a.p, b.p,
                              nullptr, nullptr),
                  "SAD atomic ROHF");
            ha = a.host(nn);
            hb = b.host(nn);
        }
        it = cache.emplace(z, std::make_pair(ha, hb)).first;
    }
    da = it->second.first;
    db = it->second.second;
}

// %g with a stream precision that switches to 17 at the first coefficient line
struct MoldenStream {
    int prec = 6;
    std::string num(double v) const
    {
        char b[64];
        std::snprintf(b, sizeof(b), "%.*g", prec, v);
        return b;
    }
};

struct OrbitalSet {
    std::string spin;
    std::vector<double> eps, C, occ;  // C row-major [basis][orbital]
};

void write_molden(const std::string& path, const Molecule& m, const std::vector<OrbitalSet>& sets)
{
    static const char shells[] = "spdfghi";
    MoldenStream st;
    std::ofstream f(path);
    if (!f) throw std::runtime_error("cannot write " + path);
    std::vector<int> nprim(m.nbf, 0), stype(m.nbf, 0);
    for (const auto& p : m.prims) {
        nprim[p.basis_index]++;
        stype[p.basis_index] = p.shell_type;
    }
    f << "[Molden Format]\ngenerated by GANSU\n[Atoms] (AU)\n";
    for (int i = 0; i < m.natom; ++i) {
        const auto& a = m.atoms[i];
        f << symbol(a.atomic_number) << " " << i + 1 << " " << a.atomic_number << " " << st.num(a.x) << " "
          << st.num(a.y) << " " << st.num(a.z) << "\n";
    }
    f << "[GTO]\n";
    const auto ranges = m.atom_ranges();
    for (int i = 0; i < m.natom; ++i) {
        f << i + 1 << " 0\n";
        for (int j = ranges[i].first; j < ranges[i].first + ranges[i].second; ++j) {
            if (nprim[j] == 0) continue;  // only the first function of a shell carries its primitives
            f << " " << shells[stype[j]] << " " << nprim[j] << " 1.00\n";
            for (const auto& p : m.prims)
                if (static_cast<int>(p.basis_index) == j) f << "\t" << st.num(p.exponent) << " " << st.num(p.coefficient) << "\n";
        }
        f << "\n";
    }
    f << "\n[MO]\n";
    const int n = m.nbf;
    for (const auto& s : sets)
        for (int i = 0; i < n; ++i) {
            f << "Sym= A\nEne= " << st.num(s.eps[i]) << "\nSpin= " << s.spin << "\nOccup= " << st.num(s.occ[i]) << "\n";
            st.prec = 17;
            for (int j = 0; j < n; ++j) f << " " << j + 1 << " " << st.num(s.C[static_cast<size_t>(j) * n + i]) << "\n";
        }
}

int guess_code(const std::string& g)
{
    if (g == "core") return HF_GUESS_CORE;
    if (g == "gwh") return HF_GUESS_GWH;
    if (g == "density") return HF_GUESS_CORE;  // no density given: the core guess (src/rhf.cu:129-132)
    if (g == "sad") return HF_GUESS_SAD;
    throw std::invalid_argument("Invalid initial guess method: " + g);
}

int run(ParameterManager& P, const std::string& dir)
{
    if (P.str("xyzfilename").empty() || P.str("gbsfilename").empty())
        throw std::invalid_argument("an xyz file (-x) and a basis set (-g) are required");
    const std::string gbs = basis_path(P.str("gbsfilename"), dir);
    const std::string method = P.str("method");
    if (method != "rhf" && method != "uhf" && method != "rohf")
        throw std::invalid_argument("Invalid method: " + method);
    Molecule m;
    check(hf_molecule_from_files(P.str("xyzfilename").c_str(), gbs.c_str(), P.integer("charge"),
                                 P.integer("beta_to_alpha"), &m.h),
          "hf_molecule_from_files");
    m.fill();
    Engine e;
    check(hf_engine_create(m.prims.data(), m.nprim, m.cgto.data(), m.nbf, m.atoms.data(), m.natom,
                           P.real("schwarz_screening_threshold"), &e.h),
          "hf_engine_create");

    hf_scf_options o;
    hf_scf_options_default(&o);
    o.max_iter = P.integer("maxiter");
    o.convergence_threshold = P.real("convergence_energy_threshold");
    o.diis_size = P.integer("diis_size");
    o.diis_include_transform = P.flag("diis_include_transform") ? 1 : 0;
    o.precision = P.str("precision") == "mixed" ? HF_PRECISION_MIXED : HF_PRECISION_FP64;
    o.mixed_threshold = P.real("mixed_threshold");
    o.verbose = P.integer("verbose");
    o.incremental = P.flag("incremental_fock") ? 1 : 0;
    o.damping_factor = P.real("damping_factor");
    const std::string conv = P.str("convergence_method");
    if (conv == "diis") o.convergence_method = HF_CONV_DIIS;
    else if (conv == "damping") o.convergence_method = HF_CONV_DAMPING;
    else if (conv == "optimaldamping") o.convergence_method = HF_CONV_OPTIMAL_DAMPING;
    else throw std::invalid_argument("Invalid convergence_method: " + conv);
    const std::string eig = P.str("eigensolver");
    o.eigensolver = eig == "purification" ? HF_EIGEN_PURIFICATION : (eig == "syevj" ? HF_EIGEN_SYEVJ : HF_EIGEN_SYEVD);
    o.initial_guess = guess_code(P.str("initial_guess"));
    const std::string eri = P.str("eri_method");
    Molecule aux;
    if (eri == "ri") {
        if (P.str("auxiliary_gbsfilename").empty()) throw std::invalid_argument("eri_method ri needs -ag");
        const std::string agbs = basis_path(P.str("auxiliary_gbsfilename"), dir);
        check(hf_molecule_from_atoms(m.atoms.data(), m.natom, agbs.c_str(), 0, 0, &aux.h), "auxiliary basis");
        aux.fill();
        check(hf_engine_set_auxiliary_basis(e.h, aux.prims.data(), aux.nprim, aux.cgto.data(), aux.nbf),
              "hf_engine_set_auxiliary_basis");
        o.eri_method = HF_ERI_RI;
    } else if (eri == "stored") {
        // ERI_Stored_RHF for RHF in FP64; the other methods and the mixed tier build directly
        o.eri_method = (method == "rhf" && o.precision == HF_PRECISION_FP64) ? HF_ERI_STORED : HF_ERI_DIRECT;
    } else if (eri == "direct") {
        o.eri_method = HF_ERI_DIRECT;
    } else {
        throw std::invalid_argument("Invalid ERI method name: " + eri);
    }

    const int n = m.nbf;
    const size_t nn = static_cast<size_t>(n) * n;
    // SAD: block-diagonal atomic densities (read_density_from_sad and the generator's atomic solves)
    DevBuf guess_a(nn), guess_b(nn);
    if (o.initial_guess == HF_GUESS_SAD) {
        std::vector<double> ha(nn, 0.0), hb(nn, 0.0), da, db;
        const auto ranges = m.atom_ranges();
        for (int i = 0; i < m.natom; ++i) {
            atomic_density(m.atoms[i].atomic_number, gbs, da, db);
            const int lo = ranges[i].first, cnt = ranges[i].second;
            if (static_cast<int>(da.size()) != cnt * cnt) throw std::runtime_error("SAD block size mismatch");
            for (int r = 0; r < cnt; ++r)
                for (int c = 0; c < cnt; ++c) {
                    ha[static_cast<size_t>(lo + r) * n + lo + c] = da[static_cast<size_t>(r) * cnt + c];
                    hb[static_cast<size_t>(lo + r) * n + lo + c] = db[static_cast<size_t>(r) * cnt + c];
                }
        }
        cuda_check(cudaMemcpy(guess_a.p, ha.data(), nn * sizeof(double), cudaMemcpyHostToDevice), "cudaMemcpy");
        cuda_check(cudaMemcpy(guess_b.p, hb.data(), nn * sizeof(double), cudaMemcpyHostToDevice), "cudaMemcpy");
        o.guess_density_a = guess_a.p;
        o.guess_density_b = guess_b.p;
    }

    hf_scf_result r;
    DevBuf Da(nn), Db(nn), eps_a(n), eps_b(n), Ca(nn), Cb(nn);
    std::vector<OrbitalSet> sets;
    const auto t0 = std::chrono::steady_clock::now();
    int st = HF_OK;
    std::string title;
    if (method == "rhf") {
        if (m.na != m.nb)
            throw std::invalid_argument(
                "In restricted Hartree Fock method, the number of alpha and beta electrons should be equal.");
        st = hf_rhf_scf(e.h, m.nel, &o, &r, Da.p, nullptr, eps_a.p, Ca.p);
        title = "Restricted Hartree-Fock (RHF)";
    } else if (method == "uhf") {
        st = hf_uhf_scf(e.h, m.na, m.nb, &o, &r, Da.p, Db.p, eps_a.p, eps_b.p, Ca.p, Cb.p);
        title = "Unrestricted Hartree-Fock (UHF)";
    } else {
        const auto& cp = rohf_couplings();
        if (!cp.count(P.str("rohf_parameter_name")))
            throw std::invalid_argument("Invalid ROHF parameter name: " + P.str("rohf_parameter_name"));
        st = hf_rohf_scf(e.h, m.na, m.nb, cp.at(P.str("rohf_parameter_name")).data(), &o, &r, Da.p, Db.p, eps_a.p,
                         Ca.p);
        title = "Restricted Open-shell Hartree-Fock (ROHF)";
    }
    const double solve_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (st != HF_OK && st != HF_ERR_NOT_CONVERGED) check(st, "SCF");

    // densities (total for the charges) and orbitals on the host
    std::vector<double> D = Da.host(nn);
    if (method != "rhf") {
        const std::vector<double> b = Db.host(nn);
        for (size_t k = 0; k < nn; ++k) D[k] += b[k];
    }
    DevBuf S(nn), H(nn);
    check(hf_compute_core_hamiltonian(e.h, S.p, H.p, nullptr), "hf_compute_core_hamiltonian");
    cuda_check(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
    const std::vector<double> Sh = S.host(nn);
    std::vector<double> occ_a(n, 0.0), occ_b(n, 0.0);
    for (int i = 0; i < n; ++i) {
        if (method == "rhf") occ_a[i] = i < m.nel / 2 ? 2.0 : 0.0;
        else if (method == "uhf") { occ_a[i] = i < m.na ? 1.0 : 0.0; occ_b[i] = i < m.nb ? 1.0 : 0.0; }
        else occ_a[i] = i < m.nb ? 2.0 : (i < m.na ? 1.0 : 0.0);
    }
    sets.push_back({"Alpha", eps_a.host(n), Ca.host(nn), occ_a});
    if (method == "uhf") sets.push_back({"Beta", eps_b.host(n), Cb.host(nn), occ_b});

    // report (HF::report, RHF::report)
    std::printf("\n");
    if (m.natom == 1) {
        std::printf("[Atom Summary]\nAtom: %s (%g, %g, %g)\n", symbol(m.atoms[0].atomic_number).c_str(), m.atoms[0].x,
                    m.atoms[0].y, m.atoms[0].z);
    } else {
        std::printf("[Molecule Summary]\nNumber of atoms: %d\n", m.natom);
        for (int i = 0; i < m.natom; ++i)
            std::printf("Atom %d: %s (%g, %g, %g)\n", i + 1, symbol(m.atoms[i].atomic_number).c_str(), m.atoms[i].x,
                        m.atoms[i].y, m.atoms[i].z);
    }
    std::printf("Number of electrons: %d\nNumber of alpha-spin electrons: %d\nNumber of beta-spin electrons: %d\n",
                m.nel, m.na, m.nb);
    std::printf("\n[Basis Set Summary]\nNumber of basis functions: %d\nNumber of primitive basis functions: %d\n",
                m.nbf, m.nprim);
    if (eri == "ri")
        std::printf("Number of auxiliary basis functions: %d\nNumber of primitive auxiliary basis functions: %d\n",
                    aux.nbf, aux.nprim);
    std::printf("\n[Charge analysis]\nMulliken population\n");
    const auto ranges = m.atom_ranges();
    for (int a = 0; a < m.natom; ++a) {
        double pop = 0.0;
        for (int i = ranges[a].first; i < ranges[a].first + ranges[a].second; ++i)
            for (int j = 0; j < n; ++j) pop += D[static_cast<size_t>(i) * n + j] * Sh[static_cast<size_t>(i) * n + j];
        std::printf("Atom %d %s: %.6g\n", a, symbol(m.atoms[a].atomic_number).c_str(), m.atoms[a].atomic_number - pop);
    }
    std::printf("\n[Calculation Summary]\nMethod: %s\n", title.c_str());
    std::printf("Schwarz screening threshold: %g\n", P.real("schwarz_screening_threshold"));
    std::printf("Initial guess method: %s\n", P.str("initial_guess").c_str());
    std::printf("Convergence algorithm: %s\n", conv.c_str());
    std::printf("Number of iterations: %d\n", r.iterations);
    std::printf("Convergence criterion: %g\n", o.convergence_threshold);
    std::printf("Converged: %s\n", r.converged ? "yes" : "no");
    std::printf("Energy (without nuclear repulsion): %.17g [hartree]\n", r.electronic_energy);
    std::printf("Total Energy: %.17g [hartree]\n", r.total_energy);
    std::printf("Computing time: %.5g [ms]\n", solve_ms);

    write_molden("output.molden", m, sets);
    if (P.flag("export_sad_cache")) {
        // HF::generate_sad_cache: N, then the alpha and beta densities (row-major, %.10e)
        std::printf("Exporting SAD cache to 'temp_sad_cache.dat'...\n");
        std::vector<double> a = Da.host(nn), b;
        if (method == "rhf") {
            for (auto& x : a) x *= 0.5;
            b = a;
        } else {
            b = Db.host(nn);
        }
        std::ofstream f("temp_sad_cache.dat");
        f << n << "\n";
        char buf[32];
        for (const auto* M : {&a, &b})
            for (int i = 0; i < n; ++i) {
                for (int j = 0; j < n; ++j) {
                    std::snprintf(buf, sizeof(buf), "%.10e ", (*M)[static_cast<size_t>(i) * n + j]);
                    f << buf;
                }
                f << "\n";
            }
        std::printf("SAD cache exported successfully.\n");
    }
    return st == HF_OK ? 0 : 1;
}

}  // namespace

int main(int argc, char** argv)
{
    ParameterManager P;
    try {
        P.parse_command_line(argc, argv, 1);
    } catch (const std::exception& ex) {
        std::fprintf(stderr, "error: %s\n", ex.what());
        return 2;
    }
    try {
        return run(P, program_dir(argv[0]));
    } catch (const std::invalid_argument& ex) {
        std::fprintf(stderr, "error: %s\n", ex.what());
        return 2;
    } catch (const std::exception& ex) {
        std::fprintf(stderr, "error: %s\n", ex.what());
        return 1;
    }
}
