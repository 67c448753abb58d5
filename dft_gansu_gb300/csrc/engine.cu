// Engine construction (the ERI plugin's precomputation).
//
//  1. contracted shells are rebuilt from the primitive list: primitives that
//     share basis_index and shell_type form one shell (the reference keeps
//     them as independent primitive shells, include/types.hpp:116-125);
//  2. shell pairs per class (la >= lb) with their primitive pairs: Gaussian
//     product data, the prefactor K and the reference's primitive Schwarz
//     bound Q = sqrt(max_comp (ab|ab)) (src/schwarz.txt:239-470), evaluated on
//     the host with the same MD templates the kernels use; the primitive
//     pairs of a shell pair are stored by bound, largest first, so the
//     kernels' primitive loops end at the first pair that fails the test;
//  3. pairs of each class sorted by Qs = sum of primitive bounds (descending),
//     so that for a bra the kets passing Qs_bra*Qs_ket >= thr form a prefix.
//     Qs >= max primitive bound, so this contracted pre-test never drops a
//     primitive quartet the reference keeps; the exact primitive test runs
//     inside the kernel;
//  4. the Boys table (F_n(k/32), n < 32) generated from the series definition.
#include <algorithm>
#include <cmath>
#include <map>
#include <memory>
#include <numeric>
#include <thread>

#include "engine.hpp"
#include "md_math.cuh"

namespace gb {

// sqrt(2 pi^{5/2}) folded into every primitive-pair prefactor K
static const double kKFold = std::sqrt(2.0 * std::pow(kPi, 2.5));

namespace {

void compute_boys_table(std::vector<double>& table)
{
    table.assign(static_cast<size_t>(kBoysRows) * kBoysPoints, 0.0);
    for (int k = 0; k < kBoysPoints; ++k)
        table[boys_exp_at(k)] = static_cast<double>(expl(-k * (long double)kBoysStep));
    const int nmax = kBoysOrders - 1;
    for (int k = 0; k < kBoysPoints; ++k) {
        const long double x = k * static_cast<long double>(kBoysStep);
        if (k == 0) {
            for (int n = 0; n <= nmax; ++n) table[boys_at(n, 0)] = 1.0 / (2 * n + 1);
            continue;
        }
        const long double ex = expl(-x);
        long double term = 1.0L / (2 * nmax + 1), sum = term;
        for (int j = 1; j < 4000; ++j) {
            term *= 2.0L * x / (2 * nmax + 2 * j + 1);
            sum += term;
            if (term < 1e-24L * sum) break;
        }
        long double f = ex * sum;
        table[boys_at(nmax, k)] = static_cast<double>(f);
        for (int n = nmax; n > 0; --n) {
            f = (2.0L * x * f + ex) / (2 * n - 1);
            table[boys_at(n - 1, k)] = static_cast<double>(f);
        }
    }
}

}  // namespace

// the table depends on nothing but the grid: computed once per process
void host_boys_table(std::vector<double>& table)
{
    static const std::vector<double> cached = [] {
        std::vector<double> t;
        compute_boys_table(t);
        return t;
    }();
    table = cached;
}

namespace {

// Diagonal (ij|ij)' of one primitive pair for all component pairs, times the
// reference's component factors; returns sqrt(max).
template <int LA, int LB>
double prim_pair_bound_t(const PrimPair64& pp, double abx, double aby, double abz, const double* boys)
{
    constexpr int NA = ncart(LA), NB = ncart(LB), L = 2 * (LA + LB), LAB = LA + LB;
    HermiteE<double, LA, LB> Ex, Ey, Ez;
    const double oo2p = 0.5 / pp.p;
    Ex.build(pp.PAx, pp.PAx + abx, oo2p);
    Ey.build(pp.PAy, pp.PAy + aby, oo2p);
    Ez.build(pp.PAz, pp.PAz + abz, oo2p);
    double Fs[L + 1];
    boys_fp64<L>(0.0, boys, Fs);
    double scale = pp.K * pp.K / (pp.p * pp.p * std::sqrt(2.0 * pp.p));
    const double m2rho = -pp.p;  // rho = p*p/(2p) = p/2, -2 rho = -p
    for (int n = 0; n <= L; ++n) { Fs[n] *= scale; scale *= m2rho; }
    HermiteR<double, L> R;
    R.build(Fs, 0.0, 0.0, 0.0);
    double mx = 0.0;
    for (int ia = 0; ia < NA; ++ia)
        for (int ib = 0; ib < NB; ++ib) {
            const int ax = cart_exp(LA, ia, 0), ay = cart_exp(LA, ia, 1), az = cart_exp(LA, ia, 2);
            const int bx = cart_exp(LB, ib, 0), by = cart_exp(LB, ib, 1), bz = cart_exp(LB, ib, 2);
            double s = 0.0;
            for (int t = 0; t <= ax + bx; ++t)
                for (int u = 0; u <= ay + by; ++u)
                    for (int v = 0; v <= az + bz; ++v) {
                        const double e1 = Ex.e[ax][bx][t] * Ey.e[ay][by][u] * Ez.e[az][bz][v];
                        for (int tau = 0; tau <= ax + bx; ++tau)
                            for (int nu = 0; nu <= ay + by; ++nu)
                                for (int phi = 0; phi <= az + bz; ++phi) {
                                    const double e2 = Ex.e[ax][bx][tau] * Ey.e[ay][by][nu] * Ez.e[az][bz][phi];
                                    const double sg = ((tau + nu + phi) & 1) ? -1.0 : 1.0;
                                    s += e1 * sg * e2 * R(t + tau, u + nu, v + phi);
                                }
                    }
            (void)LAB;
            const double cf = component_factor(LA, ia) * component_factor(LB, ib);
            mx = std::max(mx, std::fabs(s) * cf * cf);
        }
    return std::sqrt(mx);
}

// f(0) .. f(n - 1) over up to 16 host threads (static chunks); f must not share writes
template <class F>
void parallel_for(int n, const F& f)
{
    const int nt = std::max(1, std::min({n / 64, 16, static_cast<int>(std::thread::hardware_concurrency())}));
    if (nt <= 1) {
        for (int k = 0; k < n; ++k) f(k);
        return;
    }
    std::vector<std::thread> pool;
    for (int t = 0; t < nt; ++t)
        pool.emplace_back([&, t] {
            for (int k = t; k < n; k += nt) f(k);
        });
    for (auto& th : pool) th.join();
}

template <class T>
T* dev_upload(const std::vector<T>& v, int& status)
{
    T* d = nullptr;
    const size_t n = std::max<size_t>(v.size(), 1);
    cudaError_t e = cudaMalloc(&d, n * sizeof(T));
    if (e != cudaSuccess) {
        set_error(std::string("cudaMalloc: ") + cudaGetErrorString(e));
        status = (e == cudaErrorMemoryAllocation) ? HF_ERR_OUT_OF_MEMORY : HF_ERR_CUDA;
        return nullptr;
    }
    if (!v.empty()) {
        e = cudaMemcpy(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            set_error(std::string("cudaMemcpy: ") + cudaGetErrorString(e));
            status = HF_ERR_CUDA;
        }
    }
    return d;
}

template <class T>
int dev_alloc(T*& p, size_t n)
{
    cudaError_t e = cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T));
    if (e != cudaSuccess) {
        set_error(std::string("cudaMalloc: ") + cudaGetErrorString(e));
        return (e == cudaErrorMemoryAllocation) ? HF_ERR_OUT_OF_MEMORY : HF_ERR_CUDA;
    }
    return HF_OK;
}

}  // namespace

double prim_pair_bound(int la, int lb, const PrimPair64& pp, double abx, double aby, double abz, const double* boys)
{
    switch (la * 3 + lb) {
    case 0: return prim_pair_bound_t<0, 0>(pp, abx, aby, abz, boys);
    case 3: return prim_pair_bound_t<1, 0>(pp, abx, aby, abz, boys);
    case 4: return prim_pair_bound_t<1, 1>(pp, abx, aby, abz, boys);
    case 6: return prim_pair_bound_t<2, 0>(pp, abx, aby, abz, boys);
    case 7: return prim_pair_bound_t<2, 1>(pp, abx, aby, abz, boys);
    case 8: return prim_pair_bound_t<2, 2>(pp, abx, aby, abz, boys);
    default: return 0.0;
    }
}

// Primitive coefficient times the component-independent part of the
// reference's primitive norm: 2^L (2/pi)^{3/4} a^{(2L+3)/4}.
double scaled_coef(double c, double a, int L)
{
    return c * std::pow(2.0, L) * std::pow(2.0 / kPi, 0.75) * std::pow(a, (2.0 * L + 3.0) / 4.0);
}

PrimPair64 make_prim_pair(double a, double ca, const double* A, double b, double cb, const double* B)
{
    PrimPair64 r;
    const double p = a + b;
    const double ab2 = (A[0] - B[0]) * (A[0] - B[0]) + (A[1] - B[1]) * (A[1] - B[1]) + (A[2] - B[2]) * (A[2] - B[2]);
    r.p = p;
    r.invp = 1.0 / p;
    r.K = ca * cb * std::exp(-a * b / p * ab2) * kKFold;
    r.KoP = r.K / p;
    r.Q = 0.0;
    r.Px = (a * A[0] + b * B[0]) / p;
    r.Py = (a * A[1] + b * B[1]) / p;
    r.Pz = (a * A[2] + b * B[2]) / p;
    // P - A = b/p (B - A), formed from the difference to avoid cancellation
    r.PAx = b / p * (B[0] - A[0]);
    r.PAy = b / p * (B[1] - A[1]);
    r.PAz = b / p * (B[2] - A[2]);
    r.b = b;
    return r;
}

double aux_prim_bound(int l, const PrimPair64& q, const double* boys)
{
    switch (l) {
    case 0: return prim_pair_bound_t<0, 0>(q, 0.0, 0.0, 0.0, boys);
    case 1: return prim_pair_bound_t<1, 0>(q, 0.0, 0.0, 0.0, boys);
    case 2: return prim_pair_bound_t<2, 0>(q, 0.0, 0.0, 0.0, boys);
    case 3: return prim_pair_bound_t<3, 0>(q, 0.0, 0.0, 0.0, boys);
    default: return 0.0;
    }
}

Engine::~Engine()
{
    void* ptrs[] = {d_pairs,  d_pp64,   d_pp32,       d_boys64,     d_boys32,     d_scale,   d_atoms,
                    d_entry_bra, d_entry_cnt, d_entry_lo0, d_entry_prim, d_pair_qs, d_off_static, d_cp_meta, plan.off64, plan.off32,
                    plan.lo32, d_Dp64, d_Dp32, d_Jp, d_Kp, d_Jp32, d_Kp32, d_scalar, d_counters, scf.S, scf.H, scf.X, scf.F,
                    scf.D, scf.Dprev, scf.G, scf.dD, scf.C, scf.W, scf.eps, scf.T1, scf.T2, scf.E, scf.Es,
                    scf.Fs, scf.work, scf.diis, scf.J, scf.K, scf.info, scf.work_j, d_grad, d_shell_atom, d_goff64, d_goff32,
                    d_shell_info, d_block_dmax, d_mol_base, d_mol_n, d_mol_bf0, d_mol_atoms, d_shell_mol,
                    scf.P32a, scf.P32b, scf.P32c, scf.Qocc, scf.Mocc, scf.qwork, scf.qinfo, d_eri, scf.pur};
    ri_destroy(ri);
    schedule_release(sched);
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (scf.syevj_params) cusolverDnDestroySyevjInfo(scf.syevj_params);
    if (cublas) cublasDestroy(cublas);
    if (cusolver) cusolverDnDestroy(cusolver);
}


// Builds an engine over one or several molecules.  Shells, pairs and quartet
// work lists never mix molecules; matrices use the block layout of BlockMap.
int build_engine(const MolInput* mols, int nmol, double schwarz_threshold, hf_engine** out)
{
    clear_error();
    if (!mols || nmol <= 0 || !out) return set_error("build_engine: no molecules"), HF_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    int num_primitives = 0, num_basis = 0, num_atoms = 0;
    for (int m = 0; m < nmol; ++m) {
        const MolInput& M = mols[m];
        if (!M.prims || !M.cgto || !M.atoms || M.nprim <= 0 || M.nbasis <= 0 || M.natom <= 0)
            return set_error("hf_engine_create: null pointer or empty input"), HF_ERR_INVALID_ARGUMENT;
        for (int i = 0; i < M.nprim; ++i) {
            const auto& p = M.prims[i];
            if (p.shell_type < 0 || p.shell_type > kMaxL)
                return set_error("hf_engine_create: shell type " + std::to_string(p.shell_type) +
                                 " not supported (s, p, d shells)"),
                       HF_ERR_INVALID_ARGUMENT;
            if (p.basis_index + ncart(p.shell_type) > static_cast<size_t>(M.nbasis) || !(p.exponent > 0.0) ||
                p.atom_index < 0 || p.atom_index >= M.natom)
                return set_error("hf_engine_create: primitive " + std::to_string(i) + " out of range"),
                       HF_ERR_INVALID_ARGUMENT;
            if (i > 0 && M.prims[i - 1].shell_type > p.shell_type)
                return set_error("hf_engine_create: primitives must be sorted by shell type"), HF_ERR_INVALID_ARGUMENT;
        }
        num_primitives += M.nprim;
        num_basis += M.nbasis;
        num_atoms += M.natom;
    }
    auto e = std::make_unique<Engine>();
    e->num_basis = num_basis;
    e->num_atoms = num_atoms;
    e->num_prims = num_primitives;
    e->schwarz_threshold = schwarz_threshold;
    e->nmol = nmol;
    e->mol_base.assign(1, 0);
    for (int m = 0; m < nmol; ++m) {
        const MolInput& M = mols[m];
        const int bf0 = static_cast<int>(e->cgto.size()), a0 = static_cast<int>(e->atoms.size());
        e->mol_bf0.push_back(bf0);
        e->mol_n.push_back(M.nbasis);
        e->mol_atom0.push_back(a0);
        e->mol_natom.push_back(M.natom);
        e->mol_base.push_back(e->mol_base.back() + static_cast<long long>(M.nbasis) * M.nbasis);
        for (int i = 0; i < M.nprim; ++i) {
            hf_primitive_shell p = M.prims[i];
            p.basis_index += static_cast<size_t>(bf0);
            p.atom_index += a0;
            e->prims.push_back(p);
        }
        e->cgto.insert(e->cgto.end(), M.cgto, M.cgto + M.nbasis);
        e->atoms.insert(e->atoms.end(), M.atoms, M.atoms + M.natom);
    }
    e->nelem = e->mol_base.back();
    std::vector<int> atom_mol(num_atoms);
    for (int m = 0; m < nmol; ++m)
        for (int a = 0; a < e->mol_natom[m]; ++a) atom_mol[e->mol_atom0[m] + a] = m;
    const hf_primitive_shell* prims = e->prims.data();
    const hf_atom* atoms = e->atoms.data();
    e->cgto_max = *std::max_element(e->cgto.begin(), e->cgto.end());

    // ---- contracted shells: group by (shell_type, basis_index)
    std::map<std::pair<int, size_t>, std::vector<int>> groups;
    for (int i = 0; i < num_primitives; ++i) groups[{prims[i].shell_type, prims[i].basis_index}].push_back(i);
    std::vector<double> sh_alpha, sh_coef;  // scaled coefficient per shell primitive
    for (auto& kv : groups) {
        Shell s;
        s.l = kv.first.first;
        s.bf = static_cast<int>(kv.first.second);
        s.nprim = static_cast<int>(kv.second.size());
        s.prim_off = static_cast<int>(sh_alpha.size());
        const auto& p0 = prims[kv.second[0]];
        s.x = p0.x; s.y = p0.y; s.z = p0.z;
        s.atom = p0.atom_index;
        s.mol = atom_mol[p0.atom_index];
        for (int idx : kv.second) {
            sh_alpha.push_back(prims[idx].exponent);
            sh_coef.push_back(scaled_coef(prims[idx].coefficient, prims[idx].exponent, s.l));
        }
        e->shells.push_back(s);
    }
    e->num_shells = static_cast<int>(e->shells.size());
    e->scale.assign(num_basis, 0.0);
    for (const Shell& s : e->shells)
        for (int i = 0; i < ncart(s.l); ++i) e->scale[s.bf + i] = e->cgto[s.bf + i] * component_factor(s.l, i);

    std::vector<std::vector<int>> mol_shells(nmol);
    for (int i = 0; i < e->num_shells; ++i) mol_shells[e->shells[i].mol].push_back(i);

    std::vector<double> boys;
    host_boys_table(boys);

    // ---- shell pairs per class: every class's (A, B) list first, then the primitive
    // pairs and their Schwarz bounds of all of them over host threads in one pass
    // (each shell pair writes its own slice of one primitive-pair array)
    struct PairJob {
        int A, B, m, la, lb;
    };
    std::vector<PairJob> jobs;
    std::vector<int> class_job0;  // first job of each (la, lb) class, in class order
    for (int la = 0; la <= kMaxL; ++la)
        for (int lb = 0; lb <= la; ++lb) {
            class_job0.push_back(static_cast<int>(jobs.size()));
            for (int m = 0; m < nmol; ++m)
                for (int A : mol_shells[m]) {
                    if (e->shells[A].l != la) continue;
                    for (int B : mol_shells[m]) {
                        if (e->shells[B].l != lb) continue;
                        if (la == lb && B > A) continue;
                        jobs.push_back(PairJob{A, B, m, la, lb});
                    }
                }
        }
    class_job0.push_back(static_cast<int>(jobs.size()));
    std::vector<size_t> pp0(jobs.size() + 1, 0);  // slice of each shell pair in pp_all
    for (size_t k = 0; k < jobs.size(); ++k)
        pp0[k + 1] = pp0[k] + static_cast<size_t>(e->shells[jobs[k].A].nprim) * e->shells[jobs[k].B].nprim;
    std::vector<PrimPair64> pp_all(pp0.back());
    std::vector<ShellPairDev> sp_all(jobs.size());
    parallel_for(static_cast<int>(jobs.size()), [&](int k) {
        const int A = jobs[k].A, B = jobs[k].B, m = jobs[k].m, la = jobs[k].la, lb = jobs[k].lb;
        const Shell& sa = e->shells[A];
        const Shell& sb = e->shells[B];
        const double Ac[3] = {sa.x, sa.y, sa.z}, Bc[3] = {sb.x, sb.y, sb.z};
        ShellPairDev& sp = sp_all[k];
        sp = ShellPairDev{};
        sp.A = A; sp.B = B;
        sp.bfA = sa.bf - e->mol_bf0[m];  // molecule-local function indices
        sp.bfB = sb.bf - e->mol_bf0[m];
        sp.la = la; sp.lb = lb;
        sp.mbase = static_cast<int>(e->mol_base[m]);
        sp.mn = e->mol_n[m];
        sp.ABx = Ac[0] - Bc[0]; sp.ABy = Ac[1] - Bc[1]; sp.ABz = Ac[2] - Bc[2];
        PrimPair64* pp = pp_all.data() + pp0[k];
        double qs = 0.0, qm = 0.0;
        for (int i = 0; i < sa.nprim; ++i)
            for (int j = 0; j < sb.nprim; ++j) {
                PrimPair64 q = make_prim_pair(sh_alpha[sa.prim_off + i], sh_coef[sa.prim_off + i], Ac,
                                              sh_alpha[sb.prim_off + j], sh_coef[sb.prim_off + j], Bc);
                q.Q = prim_pair_bound(la, lb, q, sp.ABx, sp.ABy, sp.ABz, boys.data());
                qs += q.Q;
                qm = std::max(qm, q.Q);
                pp[i * sb.nprim + j] = q;
            }
        // largest bound first: a kernel's primitive loop over this pair ends at
        // the first primitive pair that fails the Schwarz test
        std::stable_sort(pp, pp + (pp0[k + 1] - pp0[k]),
                         [](const PrimPair64& x, const PrimPair64& y) { return x.Q > y.Q; });
        sp.Qs = qs;
        sp.Qmax = qm;
        sp.pp_n = static_cast<int>(pp0[k + 1] - pp0[k]);
    });
    e->pp64.reserve(pp_all.size());
    {
        int ci = 0;
        for (int la = 0; la <= kMaxL; ++la)
            for (int lb = 0; lb <= la; ++lb, ++ci) {
                PairClass pc{la, lb, static_cast<int>(e->pairs.size()), 0};
                // groups of equal primitive-pair count (so the lanes of a warp run
                // the same primitive loops), each group sorted by Qs descending
                std::vector<int> order;
                for (int k = class_job0[ci]; k < class_job0[ci + 1]; ++k) order.push_back(k);
                std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
                    if (jobs[a].m != jobs[b].m) return jobs[a].m < jobs[b].m;
                    if (sp_all[a].pp_n != sp_all[b].pp_n) return sp_all[a].pp_n > sp_all[b].pp_n;
                    return sp_all[a].Qs > sp_all[b].Qs;
                });
                for (size_t r = 0; r < order.size(); ++r) {
                    const int k = order[r];
                    ShellPairDev sp = sp_all[k];
                    const int mol = jobs[k].m;
                    if (r == 0 || sp_all[order[r - 1]].pp_n != sp.pp_n || jobs[order[r - 1]].m != mol) {
                        pc.groups.push_back({static_cast<int>(r), 0});
                        pc.group_mol.push_back(mol);
                    }
                    pc.groups.back().second++;
                    sp.pp_off = static_cast<int>(e->pp64.size());
                    sp.fABx = static_cast<float>(sp.ABx);
                    sp.fABy = static_cast<float>(sp.ABy);
                    sp.fABz = static_cast<float>(sp.ABz);
                    sp.fQmax = static_cast<float>(sp.Qmax);
                    e->pp64.insert(e->pp64.end(), pp_all.begin() + pp0[k], pp_all.begin() + pp0[k + 1]);
                    e->pairs.push_back(sp);
                }
                pc.count = static_cast<int>(order.size());
                e->pair_classes.push_back(pc);
            }
    }

    // ---- class pairs and bra entries (contracted pre-screen on Qs)
    const double thr = schwarz_threshold;
    // running maximum of the primitive bound Qmax over the kets of each group (kets are
    // sorted by Qs): the largest primitive bound among a group's first k kets
    std::vector<double> qmax_run(e->pairs.size());
    for (const PairClass& pc : e->pair_classes)
        for (const auto& g : pc.groups)
            for (int k = 0; k < g.second; ++k) {
                const int idx = pc.begin + g.first + k;
                qmax_run[idx] = (k == 0) ? e->pairs[idx].Qmax : std::max(qmax_run[idx - 1], e->pairs[idx].Qmax);
            }
    for (int X = 0; X < static_cast<int>(e->pair_classes.size()); ++X)
        for (int Y = 0; Y <= X; ++Y) {
            const PairClass& px = e->pair_classes[X];
            const PairClass& py = e->pair_classes[Y];
            ClassPair cp{X, Y, static_cast<int>(e->entry_bra.size()), 0, 0};
            e->off_static.push_back(0);
            long long acc = 0;
            // ket groups of each molecule (groups are sorted by molecule)
            std::vector<int> gbeg(nmol + 1, 0);
            for (size_t gi = 0; gi < py.groups.size(); ++gi) gbeg[py.group_mol[gi] + 1]++;
            for (int m = 0; m < nmol; ++m) gbeg[m + 1] += gbeg[m];
            for (int i = 0; i < px.count; ++i) {
                const double qi = e->pairs[px.begin + i].Qs;
                const int mi = e->shells[e->pairs[px.begin + i].A].mol;
                for (int gi = gbeg[mi]; gi < gbeg[mi + 1]; ++gi) {
                    const auto& g = py.groups[gi];
                    // kets of a group sorted by Qs descending: count those with qi*qj >= thr
                    int lo = 0, hi = g.second;
                    while (lo < hi) {
                        const int mid = (lo + hi) / 2;
                        if (qi * e->pairs[py.begin + g.first + mid].Qs >= thr) lo = mid + 1; else hi = mid;
                    }
                    int cnt = lo;
                    if (X == Y) cnt = std::min(cnt, i - g.first + 1);  // each unordered pair once
                    if (cnt <= 0) continue;
                    e->unique_quartets += cnt;
                    // a bra whose primitive loops are long is split over several entries, each
                    // with a range of its primitive pairs (their partial integrals are digested
                    // separately), so that no lane runs more than about kPrimPerItem primitive
                    // quartets of a quartet while the others of its warp wait
                    const ShellPairDev& bp = e->pairs[px.begin + i];
                    const int nb = bp.pp_n, nk = e->pairs[py.begin + g.first].pp_n;
                    const int nsplit = std::min(nb, std::max(1, (nb * nk + kPrimPerItem - 1) / kPrimPerItem));
                    const int chunk = (nb + nsplit - 1) / nsplit;
                    const double qket = qmax_run[py.begin + g.first + cnt - 1];  // largest among the entry's kets
                    for (int p0 = 0; p0 < nb; p0 += chunk) {
                        // a later range whose largest bound cannot pass with any ket adds nothing
                        if (p0 > 0 && e->pp64[bp.pp_off + p0].Q * qket < thr) break;
                        e->entry_bra.push_back(px.begin + i);
                        e->entry_lo0.push_back(g.first);
                        e->entry_cnt.push_back(cnt);
                        e->entry_prim.push_back(p0 | (std::min(nb, p0 + chunk) << 16));
                        acc += cnt;
                        e->off_static.push_back(acc);
                    }
                }
            }
            cp.nentry = static_cast<int>(e->entry_bra.size()) - cp.entry_begin;
            cp.n_survivors = acc;
            e->total_survivors += acc;
            e->class_pairs.push_back(cp);
        }

    // ---- device upload
    int st = HF_OK;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaFree(nullptr) != cudaSuccess)
        return set_error("hf_engine_create: no usable CUDA device"), HF_ERR_CUDA;
    cudaDeviceGetAttribute(&e->num_sms, cudaDevAttrMultiProcessorCount, dev);
    std::vector<PrimPair32> pp32(e->pp64.size());
    for (size_t i = 0; i < pp32.size(); ++i) {
        const PrimPair64& a = e->pp64[i];
        pp32[i] = PrimPair32{static_cast<float>(a.p),   static_cast<float>(a.invp), static_cast<float>(a.K),
                             static_cast<float>(a.KoP), static_cast<float>(a.Q),    static_cast<float>(a.Px),
                             static_cast<float>(a.Py),  static_cast<float>(a.Pz),   static_cast<float>(a.PAx),
                             static_cast<float>(a.PAy), static_cast<float>(a.PAz),  static_cast<float>(a.b)};
    }
    // FP32 table (boys32_at): F_n .. F_{n+3} of grid point k as one 16-byte vector
    std::vector<float> boys32(static_cast<size_t>(kBoysOrdersF) * kBoysGridF * kBoysTaylorF);
    for (int n = 0; n < kBoysOrdersF; ++n)
        for (int k = 0; k < kBoysGridF; ++k)
            for (int j = 0; j < kBoysTaylorF; ++j)
                boys32[boys32_at(n, k) + j] = static_cast<float>(boys[boys_at(n + j, k)]);
    std::vector<double> atom4(4 * num_atoms);
    for (int i = 0; i < num_atoms; ++i) {
        atom4[4 * i] = atoms[i].x; atom4[4 * i + 1] = atoms[i].y; atom4[4 * i + 2] = atoms[i].z;
        atom4[4 * i + 3] = atoms[i].atomic_number;
    }
    std::vector<double> qs(e->pairs.size());
    for (size_t i = 0; i < qs.size(); ++i) qs[i] = e->pairs[i].Qs;
    const std::vector<int>& lo0 = e->entry_lo0;
    e->d_pairs = dev_upload(e->pairs, st);
    e->d_pp64 = dev_upload(e->pp64, st);
    e->d_pp32 = dev_upload(pp32, st);
    e->d_boys64 = dev_upload(boys, st);
    e->d_boys32 = dev_upload(boys32, st);
    e->d_scale = dev_upload(e->scale, st);
    e->d_atoms = dev_upload(atom4, st);
    e->d_entry_bra = dev_upload(e->entry_bra, st);
    e->d_entry_cnt = dev_upload(e->entry_cnt, st);
    e->d_entry_lo0 = dev_upload(lo0, st);
    e->d_entry_prim = dev_upload(e->entry_prim, st);
    e->d_pair_qs = dev_upload(qs, st);
    e->d_off_static = dev_upload(e->off_static, st);
    {
        const int ncp = static_cast<int>(e->class_pairs.size());
        std::vector<int> meta(4 * ncp);
        for (int k = 0; k < ncp; ++k) {
            meta[k] = e->class_pairs[k].entry_begin;
            meta[ncp + k] = e->class_pairs[k].nentry;
            meta[2 * ncp + k] = e->pair_classes[e->class_pairs[k].Y].begin;
            meta[3 * ncp + k] = e->class_pairs[k].entry_begin + k;
        }
        e->d_cp_meta = dev_upload(meta, st);
    }
    {
        std::vector<int2> mol_atoms(nmol);
        for (int m = 0; m < nmol; ++m) mol_atoms[m] = make_int2(e->mol_atom0[m], e->mol_natom[m]);
        std::vector<int> shell_mol(e->num_shells);
        for (int i = 0; i < e->num_shells; ++i) shell_mol[i] = e->shells[i].mol;
        e->d_mol_base = dev_upload(e->mol_base, st);
        e->d_mol_n = dev_upload(e->mol_n, st);
        e->d_mol_bf0 = dev_upload(e->mol_bf0, st);
        e->d_mol_atoms = dev_upload(mol_atoms, st);
        e->d_shell_mol = dev_upload(shell_mol, st);
    }
    if (st != HF_OK) return st;
    const size_t nn = static_cast<size_t>(e->nelem);
    const size_t noff = e->off_static.size();
    if ((st = dev_alloc(e->plan.off64, noff)) || (st = dev_alloc(e->plan.off32, noff)) ||
        (st = dev_alloc(e->plan.lo32, e->entry_bra.size())) || (st = dev_alloc(e->d_Dp64, nn)) ||
        (st = dev_alloc(e->d_Dp32, nn)) || (st = dev_alloc(e->d_Jp, nn)) || (st = dev_alloc(e->d_Kp, nn)) ||
        (st = dev_alloc(e->d_Jp32, nn)) || (st = dev_alloc(e->d_Kp32, nn)) ||
        (st = dev_alloc(e->d_scalar, 16)) || (st = dev_alloc(e->d_counters, kCounterSlots)))
        return st;
    if (cudaMemset(e->d_counters, 0, kCounterSlots * sizeof(unsigned long long)) != cudaSuccess)
        return set_error("cudaMemset failed"), HF_ERR_CUDA;
    if (cublasCreate(&e->cublas) != CUBLAS_STATUS_SUCCESS) return set_error("cublasCreate failed"), HF_ERR_CUDA;
    if (cusolverDnCreate(&e->cusolver) != CUSOLVER_STATUS_SUCCESS)
        return set_error("cusolverDnCreate failed"), HF_ERR_CUDA;
    e->bytes_h2d = static_cast<long long>(
        e->pairs.size() * sizeof(ShellPairDev) + e->pp64.size() * sizeof(PrimPair64) + pp32.size() * sizeof(PrimPair32) +
        boys.size() * (sizeof(double) + sizeof(float)) + e->scale.size() * sizeof(double) + atom4.size() * sizeof(double) +
        (4 * e->entry_bra.size()) * sizeof(int) + qs.size() * sizeof(double) +
        e->off_static.size() * sizeof(long long) + 4 * e->class_pairs.size() * sizeof(int));
    *out = reinterpret_cast<hf_engine*>(e.release());
    return HF_OK;
}

}  // namespace gb

using namespace gb;

extern "C" {

int hf_engine_create(const hf_primitive_shell* prims, int num_primitives, const double* cgto_norm, int num_basis,
                     const hf_atom* atoms, int num_atoms, double schwarz_threshold, hf_engine** out)
{
    const MolInput m{prims, num_primitives, cgto_norm, num_basis, atoms, num_atoms};
    return build_engine(&m, 1, schwarz_threshold, out);
}

void hf_engine_destroy(hf_engine* eng) { delete reinterpret_cast<Engine*>(eng); }

int hf_engine_stats(const hf_engine* eng, int* num_shells, long long* num_shell_pairs, long long* num_quartets)
{
    if (!eng) return set_error("null engine"), HF_ERR_INVALID_ARGUMENT;
    const Engine* e = reinterpret_cast<const Engine*>(eng);
    if (num_shells) *num_shells = e->num_shells;
    if (num_shell_pairs) *num_shell_pairs = static_cast<long long>(e->pairs.size());
    if (num_quartets) *num_quartets = e->unique_quartets;
    return HF_OK;
}

int hf_engine_class_stats(hf_engine* eng, int max_classes, int* num_classes, int* class_l, long long* prim_fp64,
                          long long* prim_fp32, long long* contracted_fp64, long long* contracted_fp32)
{
    clear_error();
    if (!eng || !num_classes) return set_error("null argument"), HF_ERR_INVALID_ARGUMENT;
    Engine* e = reinterpret_cast<Engine*>(eng);
    const int ncp = static_cast<int>(e->class_pairs.size());
    *num_classes = ncp;
    if (max_classes < ncp) return HF_OK;
    std::vector<unsigned long long> c(kCounterSlots, 0);
    if (cudaMemcpy(c.data(), e->d_counters, kCounterSlots * sizeof(unsigned long long), cudaMemcpyDeviceToHost) !=
        cudaSuccess)
        return set_error("cudaMemcpy of counters failed"), HF_ERR_CUDA;
    for (int k = 0; k < ncp; ++k) {
        const PairClass& X = e->pair_classes[e->class_pairs[k].X];
        const PairClass& Y = e->pair_classes[e->class_pairs[k].Y];
        if (class_l) {
            class_l[4 * k] = X.la; class_l[4 * k + 1] = X.lb; class_l[4 * k + 2] = Y.la; class_l[4 * k + 3] = Y.lb;
        }
        if (prim_fp64) prim_fp64[k] = static_cast<long long>(c[4 * k + 0]);
        if (contracted_fp64) contracted_fp64[k] = static_cast<long long>(c[4 * k + 1]);
        if (prim_fp32) prim_fp32[k] = static_cast<long long>(c[4 * k + 2]);
        if (contracted_fp32) contracted_fp32[k] = static_cast<long long>(c[4 * k + 3]);
    }
    return HF_OK;
}

int hf_engine_reset_stats(hf_engine* eng)
{
    clear_error();
    if (!eng) return set_error("null argument"), HF_ERR_INVALID_ARGUMENT;
    Engine* e = reinterpret_cast<Engine*>(eng);
    if (cudaMemset(e->d_counters, 0, kCounterSlots * sizeof(unsigned long long)) != cudaSuccess)
        return set_error("cudaMemset failed"), HF_ERR_CUDA;
    return HF_OK;
}

int hf_engine_transfer_bytes(const hf_engine* eng, long long* h2d_bytes)
{
    if (!eng || !h2d_bytes) return set_error("null argument"), HF_ERR_INVALID_ARGUMENT;
    *h2d_bytes = reinterpret_cast<const Engine*>(eng)->bytes_h2d;
    return HF_OK;
}

int hf_primitive_pair_bounds(hf_engine* eng, double* h_out)
{
    clear_error();
    if (!eng || !h_out) return set_error("null argument"), HF_ERR_INVALID_ARGUMENT;
    Engine* e = reinterpret_cast<Engine*>(eng);
    std::vector<double> boys;
    host_boys_table(boys);
    const int n = e->num_prims;
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            const auto& a = e->prims[i];
            const auto& b = e->prims[j];
            // bound is symmetric in (a, b): evaluate with the higher l first
            const auto& P = (a.shell_type >= b.shell_type) ? a : b;
            const auto& Q = (a.shell_type >= b.shell_type) ? b : a;
            const double Ac[3] = {P.x, P.y, P.z}, Bc[3] = {Q.x, Q.y, Q.z};
            PrimPair64 pp = make_prim_pair(P.exponent, scaled_coef(P.coefficient, P.exponent, P.shell_type), Ac,
                                           Q.exponent, scaled_coef(Q.coefficient, Q.exponent, Q.shell_type), Bc);
            h_out[static_cast<size_t>(i) * n + j] = prim_pair_bound(P.shell_type, Q.shell_type, pp, Ac[0] - Bc[0],
                                                                    Ac[1] - Bc[1], Ac[2] - Bc[2], boys.data());
        }
    return HF_OK;
}

}  // extern "C"
