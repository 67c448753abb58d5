// Input model: Gaussian basis (.gbs) and XYZ parsers, primitive-shell
// expansion and CGTO normalisation, behind the C ABI hf_molecule_* calls.
//
// Behaviour mirrors the reference so that the same files give the same
// basis-function numbering:
//   .gbs: skip the header until the first line starting with a letter; an
//         element block is "<Sym> 0", then "<type> <nprim> <scale>" lines;
//         two-letter types (SP) split into two shells; Fortran D exponents
//         read as E; "****" ends a block        src/basis_set.cpp:32-124
//   .xyz: count, comment, "<Sym> x y z" in angstrom -> bohr x 1.8897259886,
//         near-duplicate atoms rejected         src/parseXYZ.cpp:43-119
//   basis functions numbered atom by atom, shell by shell, in file order;
//   primitive shells then sorted by shell type (the reference uses
//   std::sort; a stable sort here gives one of its valid orders)
//                                               include/molecular.hpp:117-186
//   electrons: N = sum Z - charge, alpha = ceil(N/2) + u, beta = floor(N/2) - u
//                                               include/molecular.hpp:90-109
//   CGTO factor with the reference's L/2 integer division for the second
//   primitive                                   include/basis_set.hpp:106-137
#include <algorithm>
#include <cmath>
#include <cctype>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "internal.hpp"

namespace gb {

namespace {

const char* kElements[] = {
    "H",  "He", "Li", "Be", "B",  "C",  "N",  "O",  "F",  "Ne", "Na", "Mg", "Al", "Si", "P",  "S",  "Cl", "Ar",
    "K",  "Ca", "Sc", "Ti", "V",  "Cr", "Mn", "Fe", "Co", "Ni", "Cu", "Zn", "Ga", "Ge", "As", "Se", "Br", "Kr",
    "Rb", "Sr", "Y",  "Zr", "Nb", "Mo", "Tc", "Ru", "Rh", "Pd", "Ag", "Cd", "In", "Sn", "Sb", "Te", "I",  "Xe",
    "Cs", "Ba", "La", "Ce", "Pr", "Nd", "Pm", "Sm", "Eu", "Gd", "Tb", "Dy", "Ho", "Er", "Tm", "Yb", "Lu", "Hf",
    "Ta", "W",  "Re", "Os", "Ir", "Pt", "Au", "Hg", "Tl", "Pb", "Bi", "Po", "At", "Rn"};
constexpr int kNumElements = sizeof(kElements) / sizeof(kElements[0]);

int shell_letter_to_l(char c)
{
    switch (std::toupper(static_cast<unsigned char>(c))) {
    case 'S': return 0;
    case 'P': return 1;
    case 'D': return 2;
    case 'F': return 3;
    case 'G': return 4;
    case 'H': return 5;
    case 'I': return 6;
    default: return -1;
    }
}

struct GbsShell {
    int l;
    std::vector<double> exps, coefs;
};
using GbsBasis = std::map<std::string, std::vector<GbsShell>>;

bool parse_gbs(const std::string& path, GbsBasis& out)
{
    std::ifstream ifs(path);
    if (!ifs) return set_error("cannot open basis set file: " + path), false;
    std::vector<std::string> lines;
    std::string line;
    while (std::getline(ifs, line)) {
        if (!line.empty() && line.back() == '\r') line.pop_back();
        lines.push_back(line);
    }
    size_t i = 0;
    while (i < lines.size() && !(lines[i].size() && std::isalpha(static_cast<unsigned char>(lines[i][0])))) ++i;
    while (i < lines.size()) {
        std::string elem;
        {
            std::istringstream iss(lines[i++]);
            iss >> elem;
        }
        if (elem.empty()) continue;
        std::vector<GbsShell>& shells = out[elem];
        while (i < lines.size()) {
            const std::string& hdr = lines[i++];
            if (hdr.rfind("****", 0) == 0) break;
            std::istringstream iss(hdr);
            std::string type;
            size_t nprim = 0;
            iss >> type >> nprim;
            if (type.empty()) continue;
            if (type.size() > 2) return set_error("invalid basis function name: " + type), false;
            std::vector<GbsShell> grp(type.size());
            for (size_t k = 0; k < type.size(); ++k) {
                grp[k].l = shell_letter_to_l(type[k]);
                if (grp[k].l < 0) return set_error("invalid basis function name: " + type), false;
            }
            for (size_t p = 0; p < nprim; ++p) {
                if (i >= lines.size()) return set_error("truncated basis set file: " + path), false;
                std::string row = lines[i++];
                std::replace(row.begin(), row.end(), 'D', 'E');
                std::replace(row.begin(), row.end(), 'd', 'e');
                std::istringstream rs(row);
                double e = 0;
                rs >> e;
                for (size_t k = 0; k < type.size(); ++k) {
                    double c = 0;
                    rs >> c;
                    grp[k].exps.push_back(e);
                    grp[k].coefs.push_back(c);
                }
                if (rs.fail()) return set_error("malformed primitive line in " + path + ": " + row), false;
            }
            for (auto& g : grp) shells.push_back(g);
        }
    }
    return true;
}

}  // namespace

int element_to_z(const std::string& sym)
{
    for (int z = 0; z < kNumElements; ++z)
        if (sym == kElements[z]) return z + 1;
    return -1;
}

const char* z_to_element(int z) { return (z >= 1 && z <= kNumElements) ? kElements[z - 1] : "?"; }

// CGTO factor, reference convention (include/basis_set.hpp:106-137).
double cgto_factor(int L, const std::vector<double>& a, const std::vector<double>& c)
{
    double s = 0.0;
    for (size_t i = 0; i < a.size(); ++i) {
        const double na = std::pow(2.0 * M_PI, -0.75) * std::pow(4.0 * a[i], L / 2.0 + 0.75);
        for (size_t j = 0; j < a.size(); ++j) {
            const double nb = std::pow(2.0 * M_PI, -0.75) * std::pow(4.0 * a[j], static_cast<double>(L / 2) + 0.75);
            s += c[i] * na * c[j] * nb / std::pow(2.0 * (a[i] + a[j]), L + 1.5);
        }
    }
    s *= std::pow(2.0 * M_PI, 1.5);
    return std::pow(s, -0.5);
}

int build_molecule(const std::vector<hf_atom>& atoms, const std::string& gbs_path, int charge, int beta_to_alpha,
                   Molecule& mol)
{
    if (atoms.empty()) return set_error("no atoms are given"), HF_ERR_INVALID_ARGUMENT;
    GbsBasis basis;
    if (!parse_gbs(gbs_path, basis)) return HF_ERR_IO;
    mol.atoms = atoms;
    mol.prims.clear();
    mol.cgto.clear();
    size_t bf = 0;
    for (size_t ia = 0; ia < atoms.size(); ++ia) {
        const char* sym = z_to_element(atoms[ia].atomic_number);
        auto it = basis.find(sym);
        if (it == basis.end()) return set_error(std::string("basis set does not include ") + sym), HF_ERR_IO;
        for (const GbsShell& sh : it->second) {
            for (size_t p = 0; p < sh.exps.size(); ++p) {
                hf_primitive_shell ps;
                ps.exponent = sh.exps[p];
                ps.coefficient = sh.coefs[p];
                ps.x = atoms[ia].x; ps.y = atoms[ia].y; ps.z = atoms[ia].z;
                ps.shell_type = sh.l;
                ps.basis_index = bf;
                ps.atom_index = static_cast<int>(ia);
                mol.prims.push_back(ps);
            }
            const int nc = (sh.l + 1) * (sh.l + 2) / 2;
            const double f = cgto_factor(sh.l, sh.exps, sh.coefs);
            for (int k = 0; k < nc; ++k) mol.cgto.push_back(f);
            bf += nc;
        }
    }
    mol.num_basis = static_cast<int>(bf);
    std::stable_sort(mol.prims.begin(), mol.prims.end(),
                     [](const hf_primitive_shell& a, const hf_primitive_shell& b) { return a.shell_type < b.shell_type; });
    int ne = 0;
    for (auto& a : atoms) ne += a.atomic_number;
    ne -= charge;
    if (ne < 1) return set_error("the number of electrons is less than one"), HF_ERR_INVALID_ARGUMENT;
    mol.num_electrons = ne;
    mol.num_alpha = (ne + 1) / 2 + beta_to_alpha;
    mol.num_beta = ne / 2 - beta_to_alpha;
    if (mol.num_beta < 0) return set_error("the number of beta-spin electrons is less than zero"), HF_ERR_INVALID_ARGUMENT;
    return HF_OK;
}

int parse_xyz(const std::string& path, std::vector<hf_atom>& atoms)
{
    std::ifstream ifs(path);
    if (!ifs) return set_error("failed to open xyz file: " + path), HF_ERR_IO;
    std::string line;
    if (!std::getline(ifs, line)) return set_error("failed to read atom count from file: " + path), HF_ERR_IO;
    int count = 0;
    try {
        count = std::stoi(line);
    } catch (...) {
        return set_error("invalid atom count in file: " + path), HF_ERR_IO;
    }
    if (!std::getline(ifs, line)) return set_error("failed to read comment line from file: " + path), HF_ERR_IO;
    const double a2b = 1.8897259886;
    const double dup = 1e-4;
    int lineno = 2;
    while (std::getline(ifs, line)) {
        ++lineno;
        if (!line.empty() && line.back() == '\r') line.pop_back();
        if (line.empty()) continue;
        std::istringstream iss(line);
        std::string sym;
        double x, y, z;
        if (!(iss >> sym >> x >> y >> z))
            return set_error("invalid line format in file at line " + std::to_string(lineno) + ": " + line), HF_ERR_IO;
        const int Z = element_to_z(sym);
        if (Z < 0) return set_error("unknown element symbol: " + sym), HF_ERR_IO;
        hf_atom a{Z, x * a2b, y * a2b, z * a2b};
        for (auto& e : atoms) {
            const double dx = a.x - e.x, dy = a.y - e.y, dz = a.z - e.z;
            if (dx * dx + dy * dy + dz * dz < dup * dup)
                return set_error("detected overlapping atoms at line " + std::to_string(lineno)), HF_ERR_INVALID_ARGUMENT;
        }
        atoms.push_back(a);
    }
    if (static_cast<int>(atoms.size()) != count) return set_error("atom count mismatch in file: " + path), HF_ERR_IO;
    return HF_OK;
}

}  // namespace gb

using namespace gb;

extern "C" {

int hf_molecule_from_atoms(const hf_atom* atoms, int num_atoms, const char* gbs_path, int charge, int beta_to_alpha,
                           hf_molecule** out)
{
    clear_error();
    if (!out || !gbs_path || (num_atoms > 0 && !atoms)) return set_error("null argument"), HF_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    auto* m = new Molecule();
    std::vector<hf_atom> a(atoms, atoms + std::max(num_atoms, 0));
    const int st = build_molecule(a, gbs_path, charge, beta_to_alpha, *m);
    if (st != HF_OK) {
        delete m;
        return st;
    }
    *out = reinterpret_cast<hf_molecule*>(m);
    return HF_OK;
}

int hf_molecule_from_files(const char* xyz_path, const char* gbs_path, int charge, int beta_to_alpha, hf_molecule** out)
{
    clear_error();
    if (!xyz_path || !gbs_path || !out) return set_error("null argument"), HF_ERR_INVALID_ARGUMENT;
    std::vector<hf_atom> atoms;
    const int st = parse_xyz(xyz_path, atoms);
    if (st != HF_OK) return st;
    return hf_molecule_from_atoms(atoms.data(), static_cast<int>(atoms.size()), gbs_path, charge, beta_to_alpha, out);
}

void hf_molecule_destroy(hf_molecule* mol) { delete reinterpret_cast<Molecule*>(mol); }

int hf_molecule_sizes(const hf_molecule* mol, int* num_basis, int* num_primitives, int* num_atoms, int* num_electrons,
                      int* num_alpha, int* num_beta)
{
    if (!mol) return set_error("null molecule"), HF_ERR_INVALID_ARGUMENT;
    const auto* m = reinterpret_cast<const Molecule*>(mol);
    if (num_basis) *num_basis = m->num_basis;
    if (num_primitives) *num_primitives = static_cast<int>(m->prims.size());
    if (num_atoms) *num_atoms = static_cast<int>(m->atoms.size());
    if (num_electrons) *num_electrons = m->num_electrons;
    if (num_alpha) *num_alpha = m->num_alpha;
    if (num_beta) *num_beta = m->num_beta;
    return HF_OK;
}

int hf_molecule_get(const hf_molecule* mol, hf_primitive_shell* prims, double* cgto_norm, hf_atom* atoms)
{
    if (!mol) return set_error("null molecule"), HF_ERR_INVALID_ARGUMENT;
    const auto* m = reinterpret_cast<const Molecule*>(mol);
    if (prims) std::copy(m->prims.begin(), m->prims.end(), prims);
    if (cgto_norm) std::copy(m->cgto.begin(), m->cgto.end(), cgto_norm);
    if (atoms) std::copy(m->atoms.begin(), m->atoms.end(), atoms);
    return HF_OK;
}

}  // extern "C"
