// qgpu_api.cu -- host side of the engine: descriptor validation, the batch
// layout in device memory, work tables, and the C-ABI of include/qgpu.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "qgpu_internal.cuh"

namespace {

thread_local std::string g_err;

int fail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

#define CK(call)                                                                            \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess) return fail(QGPU_E_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

template <class T>
int upload(std::vector<void *> &allocs, const std::vector<T> &h, T **d) {
    size_t n = h.size() ? h.size() : 1;
    CK(cudaMalloc((void **)d, n * sizeof(T)));
    allocs.push_back(*d);
    if (h.size()) CK(cudaMemcpy(*d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
    else CK(cudaMemset(*d, 0, sizeof(T)));
    return 0;
}
template <class T>
int alloc0(std::vector<void *> &allocs, size_t n, T **d) {
    if (!n) n = 1;
    CK(cudaMalloc((void **)d, n * sizeof(T)));
    allocs.push_back(*d);
    CK(cudaMemset(*d, 0, n * sizeof(T)));
    return 0;
}

// pad a per-trajectory segment of a work list to a multiple of QG_BLOCK
void pad(std::vector<int> &v, size_t seg_start, int traj) {
    while ((v.size() - seg_start) % QG_BLOCK) v.push_back(-1 - traj);
}

}  // namespace

// error reporting for the library's other translation units
int qgpu_fail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

struct qgpu_handle {
    int ntraj = 0;
    std::vector<TrajInfo> info;
    std::vector<int> nstates, natom, atom0, ncgp, grp0, nmol, nqat;
    std::vector<std::vector<int>> offd_states;
    DevSys S{};
    BlockTables B{};
    std::vector<void *> allocs;
    cudaStream_t stream = nullptr;
    // side streams of the per-step force kernels, which are independent of
    // one another (each adds into the fixed-point gradient and energies)
    cudaStream_t side[QG_NSIDE] = {};
    cudaEvent_t ev_fork = nullptr, ev_join[QG_NSIDE] = {};
    // Independent branches of the replayed block: groups of consecutive
    // trajectories, each with its own tables view, stream, side streams and
    // events (branch 0..nbranch-1; nbranch 1 = the whole batch on `stream`).
    int nbranch = 1;
    std::vector<BlockTables> Bg;
    cudaStream_t bstream[QG_MAXBRANCH] = {}, bside[QG_MAXBRANCH][QG_NSIDE] = {};
    cudaEvent_t bfork[QG_MAXBRANCH] = {}, bjoin[QG_MAXBRANCH][QG_NSIDE] = {}, bdone[QG_MAXBRANCH] = {};
    cudaEvent_t ev_branch = nullptr;
    // first index of every per-trajectory list, per trajectory (ntraj + 1 rows)
    struct ListStarts {
        int wgrp, satom, scan, ublk, qqblk, wp, pb, bt, qt, od, rs, xr, grp;
    };
    std::vector<ListStarts> lstart;
    long long nlaunch = 0;
    int NBcycle = 10;
    int lists_built = 0, temp_init = 0, any_shake = 0, any_wpol = 0;
    int nh_ready = 0;          // Nose-Hoover scales of the next step are formed
    std::vector<FILE *> ene_files;   // attached .en files per trajectory (or null)
    std::vector<int> fep_chain;      // trajectories of the FEP window chain
    double fep_kT = 0;
    int fep_nskip = 0;
    std::vector<char> fused;   // per trajectory: SHAKE fused into the update kernel
    bool all_fused = false;    // the fused step with the float master (QGPU_PRECISION_MIXED)
    bool fused_d = true;       // the fused step with the FP64 master (QGPU_PRECISION_FP64)
    bool can_fuse = true;      // every trajectory's constraints allow the fused update
    std::vector<int> ek_u0, ek_un, ek_a0, ek_an;   // Ekin block ranges of the two update layouts
    // 0: x/v and the float coordinates agree; 1: the float master (fused
    // steps) is newer than x/v
    int master = 0;
    long long step = 0;
    cudaGraphExec_t graph = nullptr;
    long long graph_nodes = 0;
    int graph_ene_every = 0;
    double *rec_d = nullptr;   // record rows
    int *recctl_d = nullptr;   // [0] absolute step of the block start, [1] first row of the window
    int rec_cap = 0;
    double *ecur_d = nullptr;  // one record row per trajectory for qgpu_forces
    int *zero_d = nullptr;
    double *grad_d = nullptr;
    int max_natom = 0;
    int nqt = 0;
};

// ------------------------------------------------------------- profiler
struct KernelProfiler {
    struct Rec { std::string name; cudaEvent_t a, b; };
    std::vector<Rec> recs;
    std::vector<cudaEvent_t> pool;
    cudaEvent_t get() {
        cudaEvent_t e;
        if (!pool.empty()) { e = pool.back(); pool.pop_back(); }
        else cudaEventCreate(&e);
        return e;
    }
};
void prof_begin(LaunchCtx &L, const char *name) {
    if (!L.prof) return;
    KernelProfiler::Rec r{name, L.prof->get(), L.prof->get()};
    cudaEventRecord(r.a, L.stream);
    L.prof->recs.push_back(r);
}
void prof_end(LaunchCtx &L) {
    if (!L.prof || L.prof->recs.empty()) return;
    cudaEventRecord(L.prof->recs.back().b, L.stream);
}

// ---------------------------------------------------------------- create
// Every index the device will follow is checked on the host first, so that a
// malformed descriptor is refused with QGPU_E_INVALID and never reaches a
// kernel as an out-of-range address.
static int validate_indices(const qgpu_system_desc &d, int t) {
    const int N = d.natom, S = d.nstates, nq = d.nqat;
    auto in = [](long long v, long long lo, long long hi) { return v >= lo && v < hi; };
    auto bad = [&](const char *what, long long k) {
        return fail(QGPU_E_INVALID, "traj %d: %s %lld out of range", t, what, k);
    };
    if (d.natyps < 1 || !d.avdw || !d.bvdw || !d.ljcod) return fail(QGPU_E_INVALID, "traj %d: atom type tables", t);
    for (int i = 0; i < N; ++i)
        if (!in(d.iac[i], 0, d.natyps)) return bad("atom type of atom", i);
    for (long long k = 0; k < (long long)d.natyps * d.natyps; ++k)
        if (d.ljcod[k] != 1 && d.ljcod[k] != 2) return bad("LJ code", k);
    if (d.iqatom)
        for (int i = 0; i < N; ++i)
            if (!in(d.iqatom[i], -1, nq)) return bad("Q index of atom", i);
    // charge groups
    if (d.ncgp < 1 || d.ncgp_solute < 0 || d.ncgp_solute > d.ncgp || !d.cgp_last || !d.cgp_switch || !d.cgpatom)
        return fail(QGPU_E_INVALID, "traj %d: charge groups", t);
    for (int g = 0; g < d.ncgp; ++g) {
        const int f = d.cgp_first[g], l = d.cgp_last[g];
        if (f < 0 || l < f || l >= N || !in(d.cgp_switch[g], 0, N)) return bad("charge group", g);
        for (int k = f; k <= l; ++k)
            if (!in(d.cgpatom[k], 0, N)) return bad("atom of charge group", g);
    }
    // neighbour exclusions and 1-4 pairs
    if (d.nexcl < 0 || (d.nexcl && !d.excl_pairs) || d.n14 < 0 || (d.n14 && !d.pairs14))
        return fail(QGPU_E_INVALID, "traj %d: exclusion or 1-4 lists", t);
    for (long long k = 0; k < 2LL * d.nexcl; ++k)
        if (!in(d.excl_pairs[k], 0, N)) return bad("excluded pair", k / 2);
    for (long long k = 0; k < 2LL * d.n14; ++k)
        if (!in(d.pairs14[k], 0, N)) return bad("1-4 pair", k / 2);
    // Q atoms and their lists
    if (nq > 0) {
        if (!d.iqseq || !d.qcrg || !d.qiac || d.nqlib < 1 || !d.qavdw || !d.qbvdw || !d.sc_lookup)
            return fail(QGPU_E_INVALID, "traj %d: Q-atom tables", t);
        for (int q = 0; q < nq; ++q) {
            if (!in(d.iqseq[q], 0, d.nat_solute)) return bad("atom of Q atom", q);
            for (int st = 0; st < S; ++st)
                if (!in(d.qiac[q * S + st], 0, d.nqlib)) return bad("Q type of Q atom", q);
        }
    }
    if (d.nqp14 < 0 || (d.nqp14 && !d.qp14_pairs)) return fail(QGPU_E_INVALID, "traj %d: Q 1-4 pairs", t);
    for (int k = 0; k < d.nqp14; ++k)
        if (!in(d.qp14_pairs[2 * k], 0, nq) || !in(d.qp14_pairs[2 * k + 1], 0, N)) return bad("Q 1-4 pair", k);
    long long nqq = 0;
    for (int st = 0; st < S; ++st) {
        if (d.nbqq_count[st] < 0) return bad("Q-Q pair count of state", st);
        nqq += d.nbqq_count[st];
    }
    if (nqq && (!d.nbqq_iq || !d.nbqq_j || !d.nbqq_jq || !d.nbqq_ljcod || !d.nbqq_elscale))
        return fail(QGPU_E_INVALID, "traj %d: Q-Q pair list", t);
    for (long long p = 0; p < nqq; ++p)
        if (!in(d.nbqq_iq[p], 0, nq) || !in(d.nbqq_j[p], 0, N) || !in(d.nbqq_jq[p], -1, nq) ||
            !in(d.nbqq_ljcod[p], 1, 4))
            return bad("Q-Q pair", p);
    // bonded rows: nat atoms then per-state (Q) or one (classical) code
    auto rows_ok = [&](const int32_t *rows, int n, int nat, int ncode, int code_lo, int ncod, const void *lib) {
        if (n < 0 || (n && !rows) || ncod < 0 || (ncod && !lib)) return false;
        const int w = nat + ncode;
        for (long long r = 0; r < n; ++r) {
            for (int a = 0; a < nat; ++a)
                if (!in(rows[r * w + a], 0, N)) return false;
            for (int c = 0; c < ncode; ++c)
                if (!in(rows[r * w + nat + c], code_lo, (long long)ncod + 1)) return false;
        }
        return true;
    };
    if (!rows_ok(d.qbnd, d.nqbond, 2, S, 0, d.nqbcod, d.qbondlib) ||
        !rows_ok(d.qang, d.nqangle, 3, S, 0, d.nqacod, d.qanglib) ||
        !rows_ok(d.qtor, d.nqtor, 4, S, 0, d.nqtcod, d.qtorlib) ||
        !rows_ok(d.qimp, d.nqimp, 4, S, 0, d.nqicod, d.qimplib))
        return fail(QGPU_E_INVALID, "traj %d: Q bonded terms", t);
    if (d.nbonds_solute < 0 || d.nbonds_solute > d.nbonds || d.nangles_solute < 0 || d.nangles_solute > d.nangles ||
        d.ntors_solute < 0 || d.ntors_solute > d.ntors || d.nimps_solute < 0 || d.nimps_solute > d.nimps)
        return fail(QGPU_E_INVALID, "traj %d: solute bonded counts outside 0..total", t);
    if (!rows_ok(d.bnd, d.nbonds, 2, 1, 1, d.nbndcod, d.bondlib) ||
        !rows_ok(d.ang, d.nangles, 3, 1, 1, d.nangcod, d.anglib) ||
        !rows_ok(d.tor, d.ntors, 4, 1, 1, d.ntorcod, d.torlib) ||
        !rows_ok(d.imp, d.nimps, 4, 1, 1, d.nimpcod, d.implib))
        return fail(QGPU_E_INVALID, "traj %d: bonded terms (atoms or parameter codes)", t);
    // SHAKE constraints
    if (d.shake_molecules < 0) return fail(QGPU_E_INVALID, "traj %d: shake_molecules < 0", t);
    if (d.shake_molecules > 0) {
        if (!d.shake_first || !d.shake_i || !d.shake_j || !d.shake_dist2 || d.shake_first[0] != 0)
            return fail(QGPU_E_INVALID, "traj %d: SHAKE tables", t);
        for (int m = 0; m < d.shake_molecules; ++m) {
            if (d.shake_first[m + 1] < d.shake_first[m]) return bad("SHAKE molecule", m);
            for (int c = d.shake_first[m]; c < d.shake_first[m + 1]; ++c)
                if (!in(d.shake_i[c], 0, N) || !in(d.shake_j[c], 0, N)) return bad("SHAKE constraint", c);
        }
    }
    // off-diagonal couplings: state pairs and Q-atom pairs
    if (d.noffd < 0 || (d.noffd && (!d.offd_ij || !d.offd_kl || !d.offd_Amu)))
        return fail(QGPU_E_INVALID, "traj %d: off-diagonal couplings", t);
    for (long long k = 0; k < 2LL * d.noffd; ++k)
        if (!in(d.offd_ij[k], 0, S) || !in(d.offd_kl[k], 0, nq)) return bad("off-diagonal coupling", k / 2);
    return 0;
}

static int validate(const qgpu_system_desc &d, int t) {
    if (d.natom <= 0) return fail(QGPU_E_INVALID, "traj %d: natom must be > 0", t);
    if (d.nat_solute < 0 || d.nat_solute > d.natom) return fail(QGPU_E_INVALID, "traj %d: bad nat_solute", t);
    if (d.solv_atom != 3) return fail(QGPU_E_UNSUPPORTED, "traj %d: only 3-site solvent is supported", t);
    if ((d.natom - d.nat_solute) % 3) return fail(QGPU_E_INVALID, "traj %d: solvent atoms not a multiple of 3", t);
    if (d.nwat != (d.natom - d.nat_solute) / 3)
        return fail(QGPU_E_INVALID, "traj %d: nwat %d is not the number of solvent molecules", t, d.nwat);
    if (d.ivdw_rule != 1 && d.ivdw_rule != 2)
        return fail(QGPU_E_INVALID, "traj %d: combination rule %d (1 geometric, 2 arithmetic)", t, d.ivdw_rule);
    if (d.use_pbc) {
        for (int k = 0; k < 3; ++k)
            if (!(d.boxlength[k] > 0.0)) return fail(QGPU_E_INVALID, "traj %d: box length %d not > 0", t, k);
        if (d.nqat > 0 && (d.qswitch < 0 || d.qswitch >= d.natom))
            return fail(QGPU_E_INVALID, "traj %d: Q switching atom %d outside the system", t, d.qswitch);
        if (d.Rcq < 0.0) return fail(QGPU_E_UNSUPPORTED, "traj %d: q_atom cut-off < 0 in a periodic box", t);
        if ((d.put_solute_back || d.put_solvent_back) &&
            (d.nmol < 1 || !d.istart_mol || d.nsolute_mol < 0 || d.nsolute_mol > d.nmol))
            return fail(QGPU_E_INVALID, "traj %d: molecules needed to put them back in the box", t);
        for (int m = 0; (d.put_solute_back || d.put_solvent_back) && m < d.nmol; ++m)
            if (d.istart_mol[m] < 0 || d.istart_mol[m] >= d.natom || (m && d.istart_mol[m] <= d.istart_mol[m - 1]))
                return fail(QGPU_E_INVALID, "traj %d: molecule %d start", t, m);
    }
    if (d.nstates < 1 || d.nstates > QG_MAXS)
        return fail(QGPU_E_UNSUPPORTED, "traj %d: nstates %d outside 1..%d", t, d.nstates, QG_MAXS);
    if (d.nqat < 0 || d.nqat > QG_MAXQ) return fail(QGPU_E_UNSUPPORTED, "traj %d: nqat %d > %d", t, d.nqat, QG_MAXQ);
    if (d.noffd > QG_MAXOD) return fail(QGPU_E_UNSUPPORTED, "traj %d: noffd %d > %d", t, d.noffd, QG_MAXOD);
    if (!d.x || !d.crg || !d.iac || !d.mass || !d.cgp_first) return fail(QGPU_E_INVALID, "traj %d: missing arrays", t);
    if (d.NBcycle <= 0) return fail(QGPU_E_INVALID, "traj %d: NBcycle must be > 0", t);
    if (int rc = validate_indices(d, t)) return rc;
    for (int g = d.ncgp_solute; g < d.ncgp; ++g) {
        int f = d.cgp_first[g], l = d.cgp_last[g];
        if (l - f != 2) return fail(QGPU_E_INVALID, "traj %d: solvent group %d has %d atoms", t, g, l - f + 1);
        int o = d.cgpatom[f];
        if (d.cgpatom[f + 1] != o + 1 || d.cgpatom[f + 2] != o + 2 || d.cgp_switch[g] != o || o < d.nat_solute ||
            (o - d.nat_solute) % 3)
            return fail(QGPU_E_INVALID, "traj %d: solvent group %d is not (O,H,H) in order", t, g);
    }
    for (int m = 0; m < d.shake_molecules; ++m)
        if (d.shake_first[m + 1] - d.shake_first[m] > 64)
            return fail(QGPU_E_UNSUPPORTED, "traj %d: more than 64 constraints in one molecule", t);
    for (int g = 0; g < d.ncgp; ++g)
        if (d.cgp_last[g] - d.cgp_first[g] + 1 > QG_TILE_A)
            return fail(QGPU_E_UNSUPPORTED, "traj %d: charge group %d too large", t, g);
    return 0;
}

// Ekin partial slots of each trajectory for the update kernel in use: the
// atom blocks of the fused steps (float or FP64 master), or the item blocks of
// the separate kernels (TrajInfo only; the caller uploads it).
static void set_ekin_layout(qgpu_handle *h) {
    for (int t = 0; t < h->ntraj; ++t) {
        TrajInfo &T = h->info[t];
        if (h->all_fused || h->fused_d) { T.ekin_blk0 = h->ek_a0[t]; T.ekin_nblk = h->ek_an[t]; }
        else { T.ekin_blk0 = h->ek_u0[t]; T.ekin_nblk = h->ek_un[t]; }
    }
}

// The replayed block's branches: n groups of consecutive trajectories with
// about equal atom counts, each a view of the handle's tables (pointers into
// the group's part of every per-trajectory list, and its ranges).
static void make_branches(qgpu_handle *h, int n) {
    n = std::max(1, std::min(std::min(n, QG_MAXBRANCH), h->ntraj));
    h->Bg.clear();
    h->nbranch = 1;
    if (n == 1 || h->lstart.empty()) return;
    long long tot = 0, acc = 0;
    for (int t = 0; t < h->ntraj; ++t) tot += h->natom[t];
    std::vector<int> cut{0};
    for (int t = 0; t + 1 < h->ntraj && (int)cut.size() < n; ++t) {
        acc += h->natom[t];
        if (acc * n >= tot * (long long)cut.size()) cut.push_back(t + 1);
    }
    cut.push_back(h->ntraj);
    const BlockTables &B = h->B;
    for (size_t g = 0; g + 1 < cut.size(); ++g) {
        const qgpu_handle::ListStarts &a = h->lstart[cut[g]], &b = h->lstart[cut[g + 1]];
        BlockTables V = B;
        V.wgrp = B.wgrp + a.wgrp; V.nwgrp = b.wgrp - a.wgrp;
        V.satom = B.satom + a.satom; V.nsatom = b.satom - a.satom;
        V.scan_t0 = B.scan_t0 + a.scan; V.scan_tn = B.scan_tn + a.scan; V.scan_traj = B.scan_traj + a.scan;
        V.scan_chunk = B.scan_chunk + a.scan; V.nscan = b.scan - a.scan;
        V.uatom = B.uatom + (size_t)a.ublk * QG_UBLK; V.ucon = B.ucon + (size_t)a.ublk * QG_UBLK;
        V.ublk_water = B.ublk_water + a.ublk; V.nuatom = (b.ublk - a.ublk) * QG_UBLK; V.ublk0 = a.ublk;
        V.qqblk_traj = B.qqblk_traj + a.qqblk; V.qqblk_s = B.qqblk_s + a.qqblk; V.nqqblk = b.qqblk - a.qqblk;
        if (B.nwp) { V.wp_traj = B.wp_traj + a.wp; V.wp_scr0 = B.wp_scr0 + a.wp; }
        V.nwp = b.wp - a.wp;
        if (B.npb) V.pb_traj = B.pb_traj + a.pb;
        V.npb = b.pb - a.pb;
        V.g0 = a.grp; V.ng = b.grp - a.grp;
        V.qt0 = a.qt; V.nqt = b.qt - a.qt; V.od0 = a.od; V.nod = b.od - a.od;
        V.bt0 = a.bt; V.nbtblk = b.bt - a.bt; V.rs0 = a.rs; V.nrs = b.rs - a.rs; V.xr0 = a.xr; V.nxrblk = b.xr - a.xr;
        h->Bg.push_back(V);
    }
    h->nbranch = (int)h->Bg.size();
}

static int create_impl(const qgpu_system_desc *descs, int ntraj, qgpu_handle *h) {
    h->ntraj = ntraj;
    std::vector<double> x, v, xtop, winv, mass_atom, crg_d;
    std::vector<float4> pos;
    std::vector<int> atype, aq, atraj, agrp;
    std::vector<uint8_t> aexcl, ashell, qp_skip;
    std::vector<unsigned long long> exmask, p14mask;
    std::vector<int> exl_first{0}, exl_j, exl_kind;
    std::vector<float> avdw, bvdw;
    std::vector<double> avdw_d, bvdw_d;
    std::vector<int8_t> ljcod;
    std::vector<int> g_start{0}, g_atoms, g_switch, g_kind, g_traj, tile_g0, tile_g1;
    std::vector<uint8_t> g_excl;
    std::vector<int> q_atom, qiac, qw_lj, qw_sc, qp14_first{0}, qp14_q;
    std::vector<float> ljA, ljB;
    std::vector<double> ljA_d, ljB_d;
    std::vector<float> qcrg_f, qavdw, qbvdw, sc_f, qw_A, qw_B, qwh_A, qwh_B;
    std::vector<double> qw_Ad, qw_Bd, qwh_Ad, qwh_Bd;
    std::vector<double> qcrg_d, qavdw_d, qbvdw_d, sc_d;
    std::vector<int> qq_iq, qq_j, qq_jq;
    std::vector<int8_t> qq_lj;
    std::vector<double> qq_els;
    std::vector<int> qt_atoms, qt_cod, qt_kind, qt_traj;
    std::vector<double> qt_lib;
    std::vector<int> bt_atoms, bt_cod, bt_kind, bt_blk_traj, bt_blk_slot;
    std::vector<double> bt_lib;
    std::vector<int> shk_first{0}, shk_i, shk_j, shk_traj;
    std::vector<double> shk_d2;
    std::vector<int> od_traj, od_ij, od_kl;
    std::vector<double> od_Amu;
    std::vector<int> wgrp, satom, scan_t0, scan_tn, scan_traj, scan_chunk, uitem, qqblk_traj, qqblk_s;
    // sequence restraints, water polarisation
    std::vector<int> rs_i0, rs_i1, rs_ih, rs_tc, rs_traj, wp_traj, wp_scr0;
    std::vector<int> mol_start, pb_traj;     // periodic box: molecules, put_back_in_box trajectories
    std::vector<int> xr_kind, xr_at, xr_st, xr_blk_traj;   // the other p_restrain restraints
    std::vector<double> xr_p;
    std::vector<float> xr_pf;
    std::vector<double> boxc0;
    std::vector<double> rs_fk, wp_state;
    std::vector<uint8_t> aheavy;
    long long wp_scr_n = 0;
    // thermostats: Langevin amplitudes and randm skip-ahead per atom
    std::vector<double> randva;
    std::vector<unsigned> lcg_a, lcg_c, rnd0;
    std::vector<int> uatom, ucon;
    std::vector<uint8_t> ublk_water;
    std::vector<int> ek_u0, ek_un, ek_a0, ek_an;   // Ekin block ranges of the two update layouts
    long long scr_slots = 0;
    int type0 = 0, lj0 = 0, q0 = 0, qlib0 = 0, sc0 = 0, grp0 = 0, atom0 = 0, tile0 = 0;

    for (int t = 0; t < ntraj; ++t) {
        const qgpu_system_desc &d = descs[t];
        if (int rc = validate(d, t)) return rc;
        if (t > 0 && d.NBcycle != descs[0].NBcycle)
            return fail(QGPU_E_UNSUPPORTED, "all trajectories of a batch must share NBcycle");
        h->NBcycle = d.NBcycle;
        const int N = d.natom, S = d.nstates, nq = d.nqat, nt = d.natyps;
        TrajInfo T{};
        T.atom0 = atom0; T.natom = N; T.nat_solute = d.nat_solute; T.nwat = d.nwat;
        T.grp0 = grp0; T.ncgp = d.ncgp; T.ncgp_solute = d.ncgp_solute;
        T.q0 = q0; T.nqat = nq; T.nstates = S;
        T.type0 = type0; T.natyps = nt; T.lj0 = lj0;
        T.qlib0 = qlib0; T.nqlib = d.nqlib; T.sc0 = sc0; T.qvdw = d.qvdw_flag;
        T.use_lrf = d.use_LRF; T.q_static = d.Rcq > d.rexcl_o;
        T.el14 = (float)d.el14_scale;
        T.el14d = d.el14_scale;
        T.rc2_pp = (float)(d.Rcpp * d.Rcpp); T.rc2_pw = (float)(d.Rcpw * d.Rcpw);
        T.rc2_ww = (float)(d.Rcww * d.Rcww); T.rc2_lrf = (float)(d.RcLRF * d.RcLRF);
        T.drc2_pp = d.Rcpp * d.Rcpp; T.drc2_pw = d.Rcpw * d.Rcpw; T.drc2_ww = d.Rcww * d.Rcww;
        T.drc2_lrf = d.RcLRF * d.RcLRF; T.drcq2 = d.Rcq * d.Rcq;
        for (int k = 0; k < 3; ++k) {
            T.origin[k] = d.xwcent[k]; T.xpcent[k] = d.xpcent[k]; T.xwcent[k] = d.xwcent[k];
            T.chg_solv[k] = (float)d.chg_solv[k];
        }
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) T.wwqq[3 * a + b] = (float)(d.chg_solv[a] * d.chg_solv[b]);
        T.rwat = d.rwat; T.fk_wsphere = d.fk_wsphere; T.Dwmz = d.Dwmz; T.awmz = d.awmz;
        T.fk_pshell = d.fk_pshell; T.fk_fix = d.fk_fix;
        T.fk_wspheref = (float)d.fk_wsphere; T.rwatf = (float)d.rwat; T.Dwmzf = (float)d.Dwmz; T.awmzf = (float)d.awmz;
        T.fk_pshellf = (float)d.fk_pshell; T.fk_fixf = (float)d.fk_fix;
        for (int s = 0; s < QG_MAXS; ++s) T.lambda[s] = s < S ? d.lambda[s] : 0.0;
        for (int s = 0; s < QG_MAXS; ++s) T.lambdaf[s] = (float)T.lambda[s];
        T.dt = d.dt; T.Temp0 = d.Temp0; T.tau_T = d.tau_T; T.inv_dt = 1.0 / d.dt;
        T.dtf = (float)T.dt; T.inv_dtf = (float)T.inv_dt;
        {
            const double boltz = 0.001986;   // src/md.f90:54
            auto c = [&](int n) { return n > 0 ? (float)(2.0 / boltz / (double)n) : 0.f; };
            T.cT = c(d.Ndegf); T.cTfree = c(d.Ndegfree);
            T.cTfsu = c(d.Ndegfree_solute); T.cTfsv = c(d.Ndegfree_solvent);
            T.dt_tau = (float)(d.dt / d.tau_T); T.Temp0f = (float)d.Temp0;
            T.dt_taud = d.dt / d.tau_T;
        }
        T.separate_scaling = d.separate_scaling; T.detail_temps = d.detail_temps;
        T.any_atom = d.any_atom_lists ? 1 : 0;
        // --- periodic box (the Q lists follow the switching atom: rebuilt with every list)
        for (int k = 0; k < 3; ++k) boxc0.push_back(d.use_pbc ? d.boxcentre[k] : 0.0);
        if (d.use_pbc) {
            T.pbc = 1; T.q_static = 0;
            T.qswitch = nq > 0 ? atom0 + d.qswitch : -1;
            for (int k = 0; k < 3; ++k) {
                T.box[k] = d.boxlength[k]; T.ibox[k] = 1.0 / d.boxlength[k];
                T.boxf[k] = (float)T.box[k]; T.iboxf[k] = (float)T.ibox[k];
            }
            T.put_solute = d.put_solute_back; T.put_solvent = d.put_solvent_back;
            T.rigid_box = d.rigid_box_centre;
            if (d.put_solute_back || d.put_solvent_back) {
                T.mol0 = (int)mol_start.size(); T.nmol = d.nmol; T.nsolute_mol = d.nsolute_mol;
                for (int m = 0; m < d.nmol; ++m) mol_start.push_back(atom0 + d.istart_mol[m]);
                mol_start.push_back(atom0 + N);
                pb_traj.push_back(t);
            }
        }
        T.Ndegf = d.Ndegf; T.Ndegfree = d.Ndegfree;
        T.Ndegfree_solute = d.Ndegfree_solute; T.Ndegfree_solvent = d.Ndegfree_solvent;
        T.ff_type = d.ff_type;
        // --- sequence restraints (p_restrain, src/md.f90:15484-15576)
        for (int r = 0; r < d.nrstr_seq; ++r) {
            const int a = d.rstseq_ij[2 * r], b = d.rstseq_ij[2 * r + 1];
            if (a < 0 || b >= N || a > b) return fail(QGPU_E_INVALID, "trajectory %d: sequence restraint %d atoms", t, r);
            rs_i0.push_back(atom0 + a); rs_i1.push_back(atom0 + b);
            rs_fk.push_back(d.rstseq_fk[r]); rs_ih.push_back(d.rstseq_flags[2 * r]);
            rs_tc.push_back(d.rstseq_flags[2 * r + 1]); rs_traj.push_back(t);
        }
        for (int i = 0; i < N; ++i)
            aheavy.push_back(d.heavy ? d.heavy[i] : (uint8_t)(d.mass[d.iac[i]] >= 4.0));
        // --- the other p_restrain restraints (src/md.f90:15580-15800), one item
        // each (a wall restraint one per selected atom), padded to QG_BLOCK
        {
            const size_t n0 = xr_kind.size();
            auto item = [&](int kind, int i, int j, int k, int st, const double *p, int np) {
                xr_kind.push_back(kind);
                xr_at.push_back(atom0 + i); xr_at.push_back(atom0 + j); xr_at.push_back(atom0 + k);
                xr_st.push_back(st);
                for (int q = 0; q < 6; ++q) xr_p.push_back(q < np ? p[q] : 0.0);
                float f[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
                if (kind == 0) {
                    for (int a = 0; a < 3; ++a) {
                        const double r = p[a] - d.xwcent[a];
                        f[a] = (float)r;
                        f[3 + a] = (float)(r - (double)f[a]);
                        f[6 + a] = (float)p[3 + a];
                    }
                } else {
                    for (int q = 0; q < np; ++q) f[q] = (float)p[q];
                }
                for (int q = 0; q < 9; ++q) xr_pf.push_back(f[q]);
            };
            auto bad = [&](int a) { return a < 0 || a >= N; };
            auto bad_st = [&](int st) { return st < 0 || st > S; };
            for (int r = 0; r < d.nrstr_pos; ++r) {
                const int i = d.rstpos_i[2 * r], st = d.rstpos_i[2 * r + 1];
                if (bad(i) || bad_st(st)) return fail(QGPU_E_INVALID, "trajectory %d: atom restraint %d", t, r);
                item(0, i, i, i, st, d.rstpos_x + 6 * r, 6);
            }
            for (int r = 0; r < d.nrstr_dist; ++r) {
                const int i = d.rstdis_i[3 * r], j = d.rstdis_i[3 * r + 1], st = d.rstdis_i[3 * r + 2];
                if (bad(i) || bad(j) || bad_st(st)) return fail(QGPU_E_INVALID, "trajectory %d: distance restraint %d", t, r);
                item(1, i, j, j, st, d.rstdis_p + 3 * r, 3);
            }
            for (int r = 0; r < d.nrstr_angl; ++r) {
                const int i = d.rstang_i[4 * r], j = d.rstang_i[4 * r + 1], k = d.rstang_i[4 * r + 2];
                const int st = d.rstang_i[4 * r + 3];
                if (bad(i) || bad(j) || bad(k) || bad_st(st))
                    return fail(QGPU_E_INVALID, "trajectory %d: angle restraint %d", t, r);
                item(2, i, j, k, st, d.rstang_p + 2 * r, 2);
            }
            for (int r = 0; r < (d.use_pbc ? 0 : d.nrstr_wall); ++r) {
                const int a0 = d.rstwal_i[3 * r], a1 = d.rstwal_i[3 * r + 1], ih = d.rstwal_i[3 * r + 2];
                if (bad(a0) || bad(a1) || a0 > a1) return fail(QGPU_E_INVALID, "trajectory %d: wall restraint %d", t, r);
                for (int i = a0; i <= a1; ++i) {
                    const bool heavy = d.heavy ? d.heavy[i] : d.mass[d.iac[i]] >= 4.0;
                    if (heavy || ih == 1) item(3, i, i, i, 0, d.rstwal_p + 4 * r, 4);
                }
            }
            const size_t n = xr_kind.size() - n0;
            if (n) {
                const double zero6[6] = {0, 0, 0, 0, 0, 0};
                while ((xr_kind.size() - n0) % QG_BLOCK) {
                    item(0, 0, 0, 0, 0, zero6, 6);
                    xr_kind.back() = -1;
                }
                for (size_t b = 0; b < (xr_kind.size() - n0) / QG_BLOCK; ++b) xr_blk_traj.push_back(t);
            }
        }
        T.freeze = d.excluded_freeze;
        // --- thermostat / integrator (md_run :6440-6460)
        if (d.thermostat < 0 || d.thermostat > 2 || d.integrator < 0 || d.integrator > 1)
            return fail(QGPU_E_INVALID, "trajectory %d: thermostat %d / integrator %d", t, d.thermostat, d.integrator);
        if (d.thermostat == 2 && (d.nhchains < 1 || d.nhchains > QG_MAXNH))
            return fail(QGPU_E_UNSUPPORTED, "trajectory %d: Nose-Hoover chain of %d (1..%d)", t, d.nhchains, QG_MAXNH);
        T.thermostat = d.thermostat; T.integrator = d.integrator; T.lgauss = d.langevin_gauss ? 1 : 0;
        T.dvm = d.integrator == 1 ? 0.5 * d.dt : d.dt;
        T.dvmf = (float)T.dvm;
        T.dvm_q = T.dvm * (1.0 / QG_FSCALE);
        T.lfric = 1.0 - d.friction * T.dvm;
        T.lfricf = (float)T.lfric;
        T.kbT = 0.001986 * d.Temp0;
        T.nhc = d.thermostat == 2 ? d.nhchains : 0;
        for (int c = 0; c < T.nhc; ++c) T.qnh[c] = c == 0 ? d.Ndegf * d.nhq : d.nhq;
        {
            // x_{n+k} = A_k x_n + C_k (mod 10^8) for the randm stream
            const unsigned long long m = QG_LCG_M;
            auto comp = [&](unsigned long long a1, unsigned long long c1, unsigned long long &a, unsigned long long &c) {
                c = (a1 * c + c1) % m;   // apply (a1, c1) after (a, c)
                a = (a1 * a) % m;
            };
            const int per = d.langevin_gauss ? 36 : 3;
            unsigned long long ap = 1, cp = 0;
            for (int q = 0; q < per; ++q) comp(QG_LCG_MULT, 1, ap, cp);
            unsigned long long a = 1, c = 0;
            const double gk = (d.langevin_gauss ? 2.0 : 24.0) * d.friction * 0.001986 * d.Temp0 / T.dvm;
            for (int i = 0; i < N; ++i) {
                lcg_a.push_back((unsigned)a); lcg_c.push_back((unsigned)c);
                randva.push_back(d.thermostat == 1 ? sqrt(gk * d.mass[d.iac[i]]) : 0.0);
                comp(ap, cp, a, c);
            }
            T.lcgA = a; T.lcgC = c;
            rnd0.push_back((unsigned)(std::abs((long long)d.rand_state) % (long long)m));
        }
        // --- water polarisation shells (watpol, wat_shells)
        T.wp0 = (int)(wp_state.size() / 3);
        if (d.wpol_restr && d.nwat > 0 && d.nwpolr_shell > 0) {
            if (!d.wshell_rout || !d.wshell_dr || !d.wshell_cstb || !d.wshell_theta_corr)
                return fail(QGPU_E_INVALID, "trajectory %d: polarisation shell tables", t);
            if (d.nwpolr_shell > QG_MAXSHELL)
                return fail(QGPU_E_UNSUPPORTED, "trajectory %d: %d polarisation shells (max %d)", t, d.nwpolr_shell,
                            QG_MAXSHELL);
            T.wpol = 1; T.nshell = d.nwpolr_shell; T.fkwpol = d.fkwpol; T.itdis_update = d.itdis_update;
            for (int k = 0; k < d.nwpolr_shell; ++k) {
                T.sh_rout[k] = d.wshell_rout[k]; T.sh_cstb[k] = d.wshell_cstb[k];
                T.sh_acos_cstb[k] = acos(d.wshell_cstb[k]);
                wp_state.push_back(d.wshell_theta_corr ? d.wshell_theta_corr[k] : 0.0);
                wp_state.push_back(0.0); wp_state.push_back(0.0);
            }
            T.wp_rlayer = d.wshell_rout[d.nwpolr_shell - 1] - d.wshell_dr[d.nwpolr_shell - 1];
            wp_traj.push_back(t); wp_scr0.push_back((int)wp_scr_n);
            wp_scr_n += (28LL * d.nwat + 4) / 8 + 2;
        }
        // --- types
        for (int a = 0; a < nt; ++a)
            for (int c = 0; c < 3; ++c) {
                avdw.push_back((float)d.avdw[a * 3 + c]); bvdw.push_back((float)d.bvdw[a * 3 + c]);
                avdw_d.push_back(d.avdw[a * 3 + c]); bvdw_d.push_back(d.bvdw[a * 3 + c]);
            }
        for (int k = 0; k < nt * nt; ++k) ljcod.push_back(d.ljcod[k]);
        // --- LJ products per (type pair, code): geometric A = a_i a_j,
        // B = b_i b_j; arithmetic (nonbon2_pp :11354, nonbon2_pw :11569)
        // A = b_i b_j (a_i + a_j)^12, B = 2 b_i b_j (a_i + a_j)^6
        T.arith = d.ivdw_rule == 2 ? 1 : 0;
        auto arith_ab = [](double ai, double aj, double bi, double bj, double &A, double &B) {
            double a = ai + aj;
            a = a * a;
            a = a * a * a;
            const double b = bi * bj;
            A = b * a * a;
            B = 2.0 * b * a;
        };
        for (int ta = 0; ta < nt; ++ta)
            for (int tb = 0; tb < nt; ++tb)
                for (int c = 0; c < 3; ++c) {
                    double A, B;
                    if (T.arith) arith_ab(d.avdw[ta * 3 + c], d.avdw[tb * 3 + c], d.bvdw[ta * 3 + c], d.bvdw[tb * 3 + c], A, B);
                    else { A = d.avdw[ta * 3 + c] * d.avdw[tb * 3 + c]; B = d.bvdw[ta * 3 + c] * d.bvdw[tb * 3 + c]; }
                    ljA.push_back((float)A); ljB.push_back((float)B);
                    ljA_d.push_back(A); ljB_d.push_back(B);
                }
        // --- water LJ constants (nonbond_ww_spc uses aLJ_solv(1,iLJ)^2;
        // nonbon2_ww :12847 the arithmetic form of the O pair)
        if (d.nwat > 0) {
            int tO = d.iac[d.nat_solute];
            int c = d.ljcod[tO * nt + tO];
            T.ww_lj = c;
            double A = d.aLJ_solv[c - 1] * d.aLJ_solv[c - 1], B = d.bLJ_solv[c - 1] * d.bLJ_solv[c - 1];
            if (T.arith) arith_ab(d.aLJ_solv[c - 1], d.aLJ_solv[c - 1], d.bLJ_solv[c - 1], d.bLJ_solv[c - 1], A, B);
            T.ww_A = (float)A; T.ww_B = (float)B;
            T.ww_Ad = A; T.ww_Bd = B;
            // arithmetic rule: nonbon2_ww (:12847-12944) takes LJ on all nine
            // atom pairs, (a_i + a_j)^6 and b_i b_j of aLJ_solv / bLJ_solv with
            // each pair's own LJ code; the eight pairs beside O-O are the
            // extra kernel's when some hydrogen carries LJ
            T.hlj = 0;
            for (int k = 0; k < 9; ++k) { T.wwh_A[k] = T.wwh_B[k] = 0.f; T.wwh_Ad[k] = T.wwh_Bd[k] = 0.0; }
            if (T.arith && (d.bLJ_solv[2] != 0.0 || d.bLJ_solv[3] != 0.0 || d.bLJ_solv[4] != 0.0 ||
                            d.bLJ_solv[5] != 0.0)) {
                T.hlj = 1;
                for (int a = 0; a < 3; ++a)
                    for (int b = 0; b < 3; ++b) {
                        if (a == 0 && b == 0) continue;
                        const int ta = d.iac[d.nat_solute + a], tb = d.iac[d.nat_solute + b];
                        const int cc = d.ljcod[ta * nt + tb];
                        double Ah, Bh;
                        arith_ab(d.aLJ_solv[a * 2 + cc - 1], d.aLJ_solv[b * 2 + cc - 1], d.bLJ_solv[a * 2 + cc - 1],
                                 d.bLJ_solv[b * 2 + cc - 1], Ah, Bh);
                        T.wwh_A[3 * a + b] = (float)Ah; T.wwh_B[3 * a + b] = (float)Bh;
                        T.wwh_Ad[3 * a + b] = Ah; T.wwh_Bd[3 * a + b] = Bh;
                    }
                T.wh_col[0] = d.iac[d.nat_solute + 1];
                T.wh_col[1] = d.iac[d.nat_solute + 2];
            }
        } else { T.ww_lj = 1; T.hlj = 0; }
        // --- atoms
        std::vector<int> grp_of(N, 0);
        for (int g = 0; g < d.ncgp; ++g)
            for (int k = d.cgp_first[g]; k <= d.cgp_last[g]; ++k) grp_of[d.cgpatom[k]] = g;
        for (int i = 0; i < N; ++i) {
            for (int c = 0; c < 3; ++c) {
                x.push_back(d.x[3 * i + c]);
                v.push_back(d.v ? d.v[3 * i + c] : 0.0);
                xtop.push_back(d.xtop ? d.xtop[3 * i + c] : d.x[3 * i + c]);
            }
            double m = d.mass[d.iac[i]];
            winv.push_back(1.0 / m);
            mass_atom.push_back(m);
            crg_d.push_back(d.crg[i]);
            pos.push_back(make_float4(0, 0, 0, (float)d.crg[i]));
            atype.push_back(type0 + d.iac[i]);
            aq.push_back(d.iqatom[i] >= 0 ? q0 + d.iqatom[i] : -1);
            atraj.push_back(t);
            agrp.push_back(grp0 + grp_of[i]);
            aexcl.push_back(d.excl ? d.excl[i] : 0);
            ashell.push_back(d.shell ? d.shell[i] : 0);
            qp_skip.push_back(d.qp_skip ? d.qp_skip[i] : 0);
        }
        // exclusion masks (offset -32..31) and long pairs, both directions
        std::vector<unsigned long long> em(N, 0ull), pm(N, 0ull);
        std::vector<std::vector<std::pair<int, int>>> lng(N);
        auto put = [&](const int32_t *pr, int np, int kind) {
            for (int k = 0; k < np; ++k) {
                int a = pr[2 * k], b = pr[2 * k + 1];
                for (int dir = 0; dir < 2; ++dir) {
                    int i = dir ? b : a, j = dir ? a : b, rel = j - i;
                    if (rel >= -32 && rel < 32) (kind ? pm : em)[i] |= 1ull << (rel + 32);
                    else lng[i].push_back({j, kind});
                }
            }
        };
        put(d.excl_pairs, d.nexcl, 0);
        put(d.pairs14, d.n14, 1);
        for (int i = 0; i < N; ++i) {
            exmask.push_back(em[i]); p14mask.push_back(pm[i]);
            for (auto &p : lng[i]) { exl_j.push_back(atom0 + p.first); exl_kind.push_back(p.second); }
            exl_first.push_back((int)exl_j.size());
        }
        // --- groups and scan tiles
        T.tile0 = tile0;
        int tg0 = grp0, tat = 0, tng = 0;
        for (int g = 0; g < d.ncgp; ++g) {
            int na = d.cgp_last[g] - d.cgp_first[g] + 1;
            if (tng == QG_TILE_G || tat + na > QG_TILE_A) {
                tile_g0.push_back(tg0); tile_g1.push_back(grp0 + g); tile0++;
                tg0 = grp0 + g; tat = 0; tng = 0;
            }
            tat += na; tng++;
            for (int k = d.cgp_first[g]; k <= d.cgp_last[g]; ++k) g_atoms.push_back(atom0 + d.cgpatom[k]);
            g_start.push_back((int)g_atoms.size());
            g_switch.push_back(atom0 + d.cgp_switch[g]);
            g_kind.push_back(g >= d.ncgp_solute ? 1 : 0);
            g_excl.push_back(d.excl ? d.excl[d.cgp_switch[g]] : 0);
            g_traj.push_back(t);
        }
        if (tng) { tile_g0.push_back(tg0); tile_g1.push_back(grp0 + d.ncgp); tile0++; }
        T.ntile = tile0 - T.tile0;
        T.nchunk = (T.ntile + QG_TPC - 1) / QG_TPC;
        T.scr0 = scr_slots;
        scr_slots += (long long)T.nchunk * d.ncgp;
        for (int b = 0; b < d.ncgp; b += QG_BLOCK)
            for (int c = 0; c < T.nchunk; ++c) {
                scan_t0.push_back(grp0 + b); scan_tn.push_back(std::min(QG_BLOCK, d.ncgp - b));
                scan_traj.push_back(t); scan_chunk.push_back(c);
            }
        // --- work lists
        size_t s0 = wgrp.size();
        {
            // water work order: by 1 A shells of the distance from the solvent
            // centre, inner first (neighbour counts fall towards the surface,
            // so a warp's lane groups get similar loads), topology order inside
            // a shell.  The order changes no result: each water sums its own
            // pairs and the block sums are fixed point.
            std::vector<std::pair<int, int>> key;
            for (int g = d.ncgp_solute; g < d.ncgp; ++g) {
                const int o = d.cgp_switch[g];
                double r2 = 0;
                for (int c = 0; c < 3; ++c) {
                    const double dx = d.x[3 * o + c] - d.xwcent[c];
                    r2 += dx * dx;
                }
                key.push_back({(int)std::sqrt(r2), g});
            }
            std::stable_sort(key.begin(), key.end(),
                             [](const std::pair<int, int> &a, const std::pair<int, int> &b) { return a.first < b.first; });
            for (const auto &k : key) wgrp.push_back(grp0 + k.second);
        }
        pad(wgrp, s0, t);
        s0 = satom.size();
        for (int i = 0; i < d.nat_solute; ++i) satom.push_back(atom0 + i);
        pad(satom, s0, t);
        // update items: 3-atom molecules whose constraints stay inside (O,H,H)
        // are updated and shaken by one thread; every other atom on its own
        {
            bool fuse = true;
            for (int m = 0; m < d.shake_molecules && fuse; ++m) {
                int c0 = d.shake_first[m], c1 = d.shake_first[m + 1];
                int lo = d.natom, hi = -1;
                for (int c = c0; c < c1; ++c) {
                    lo = std::min(lo, std::min(d.shake_i[c], d.shake_j[c]));
                    hi = std::max(hi, std::max(d.shake_i[c], d.shake_j[c]));
                }
                // fused only for the water pattern O-H1, O-H2, H1-H2 in this order
                if (c1 - c0 != 3 || hi - lo != 2 ||
                    d.shake_i[c0] != lo || d.shake_j[c0] != lo + 1 ||
                    d.shake_i[c0 + 1] != lo || d.shake_j[c0 + 1] != lo + 2 ||
                    d.shake_i[c0 + 2] != lo + 1 || d.shake_j[c0 + 2] != lo + 2)
                    fuse = false;
            }
            std::vector<int> owner(N, -1);
            if (fuse)
                for (int m = 0; m < d.shake_molecules; ++m) {
                    int lo = d.shake_i[d.shake_first[m]];
                    for (int k = 0; k < 3 && lo + k < N; ++k) {
                        if (owner[lo + k] >= 0) fuse = false;
                        owner[lo + k] = m;
                    }
                }
            // the fused update writes the packed water records only in its
            // water blocks: every water must be one of them
            if (fuse)
                for (int i = d.nat_solute; i < N; ++i)
                    if (owner[i] < 0) fuse = false;
            h->fused.push_back(fuse);
            s0 = uitem.size();
            T.ekin_blk0 = (int)(uitem.size() / QG_BLOCK);
            int shk_base = (int)(shk_first.size() - 1);
            for (int i = 0; i < N; ++i) {
                if (fuse && owner[i] >= 0) {
                    if (d.shake_i[d.shake_first[owner[i]]] == i) uitem.push_back((1 << 30) | (shk_base + owner[i]));
                } else uitem.push_back(atom0 + i);
            }
            pad(uitem, s0, t);
            T.ekin_nblk = (int)((uitem.size() - s0) / QG_BLOCK);
            ek_u0.push_back(T.ekin_blk0); ek_un.push_back(T.ekin_nblk);
            // atom layout of the fused update
            const size_t u0 = uatom.size();
            auto upad = [&]() {
                while ((uatom.size() - u0) % QG_UBLK) { uatom.push_back(-1 - t); ucon.push_back(-1); }
            };
            for (int i = 0; i < N; ++i)
                if (!(fuse && owner[i] >= 0)) { uatom.push_back(atom0 + i); ucon.push_back(-1); }
            upad();
            const size_t nb_plain = (uatom.size() - u0) / QG_UBLK;
            if (fuse) {
                const int cbase = (int)shk_i.size();   // this trajectory's constraints come next
                for (int m = 0; m < d.shake_molecules; ++m) {
                    const int lo = d.shake_i[d.shake_first[m]];
                    for (int k = 0; k < 3; ++k) {
                        uatom.push_back(atom0 + lo + k);
                        ucon.push_back(k == 0 ? cbase + d.shake_first[m] : -1);
                    }
                }
                upad();
            }
            const size_t nb_all = (uatom.size() - u0) / QG_UBLK;
            for (size_t b = 0; b < nb_all; ++b) ublk_water.push_back(b >= nb_plain ? 1 : 0);

            ek_a0.push_back((int)(u0 / QG_UBLK)); ek_an.push_back((int)nb_all);
        }
        // --- Q atoms
        int nql = d.nqlib;
        for (int k = 0; k < nql; ++k)
            for (int c = 0; c < 3; ++c) {
                qavdw.push_back((float)d.qavdw[k * 3 + c]); qbvdw.push_back((float)d.qbvdw[k * 3 + c]);
                qavdw_d.push_back(d.qavdw[k * 3 + c]); qbvdw_d.push_back(d.qbvdw[k * 3 + c]);
            }
        int tO = d.nwat > 0 ? d.iac[d.nat_solute] : 0;
        for (int iq = 0; iq < nq; ++iq) {
            int qa = d.iqseq[iq];
            q_atom.push_back(atom0 + qa);
            int tq = d.iac[qa];
            int c = d.ljcod[tO * nt + tq];
            qw_lj.push_back(c);
            // softcore column of the O: the LJ code (nonbond_qw_spc :14492), its
            // type for the arithmetic rule (nonbon2_qw :12632)
            qw_sc.push_back(T.arith ? tO : c - 1);
            for (int s = 0; s < QG_MAXS; ++s) {
                double qc = s < S ? d.qcrg[iq * S + s] : 0.0;
                qcrg_d.push_back(qc); qcrg_f.push_back((float)qc);
                int qt = s < S ? d.qiac[iq * S + s] : 0;
                qiac.push_back(qlib0 + qt);
                double A, B;
                if (T.arith) {
                    // nonbon2_qw: (a_q + a_O)^6, b_q b_O with the Q atom's type or
                    // its state's Q type (code 2 -> 1)
                    const int cq = c == 2 ? 1 : c;
                    const double aq = d.qvdw_flag ? d.qavdw[qt * 3 + cq - 1] : d.avdw[tq * 3 + c - 1];
                    const double bq = d.qvdw_flag ? d.qbvdw[qt * 3 + cq - 1] : d.bvdw[tq * 3 + c - 1];
                    arith_ab(aq, d.aLJ_solv[c - 1], bq, d.bLJ_solv[c - 1], A, B);
                } else if (!d.qvdw_flag) {
                    A = d.avdw[tq * 3 + c - 1] * d.aLJ_solv[c - 1];
                    B = d.bvdw[tq * 3 + c - 1] * d.bLJ_solv[c - 1];
                } else {
                    A = d.qavdw[qt * 3] * d.aLJ_solv[c - 1];
                    B = d.qbvdw[qt * 3] * d.bLJ_solv[c - 1];
                }
                qw_A.push_back((float)A); qw_B.push_back((float)B);
                qw_Ad.push_back(A); qw_Bd.push_back(B);
                // nonbon2_qw with the two water hydrogens: aLJ_solv / bLJ_solv of
                // the H and the LJ code of the (H, Q atom) pair
                for (int h = 0; h < 2; ++h) {
                    double Ah = 0.0, Bh = 0.0;
                    if (T.hlj) {
                        const int tH = d.iac[d.nat_solute + 1 + h];
                        const int ch = d.ljcod[tH * nt + tq], cq = ch == 2 ? 1 : ch;
                        const double aq = d.qvdw_flag ? d.qavdw[qt * 3 + cq - 1] : d.avdw[tq * 3 + ch - 1];
                        const double bq = d.qvdw_flag ? d.qbvdw[qt * 3 + cq - 1] : d.bvdw[tq * 3 + ch - 1];
                        arith_ab(aq, d.aLJ_solv[(1 + h) * 2 + ch - 1], bq, d.bLJ_solv[(1 + h) * 2 + ch - 1], Ah, Bh);
                    }
                    qwh_A.push_back((float)Ah); qwh_B.push_back((float)Bh);
                    qwh_Ad.push_back(Ah); qwh_Bd.push_back(Bh);
                }
            }
        }
        int ntq = nt + nq;
        for (int iq = 0; iq < nq; ++iq)
            for (int col = 0; col < ntq; ++col)
                for (int s = 0; s < QG_MAXS; ++s) {
                    double sc = (s < S && d.sc_lookup) ? d.sc_lookup[((size_t)iq * ntq + col) * S + s] : 0.0;
                    sc_d.push_back(sc); sc_f.push_back((float)sc);
                }
        {
            std::vector<std::vector<int>> q14(N);
            for (int k = 0; k < d.nqp14; ++k) q14[d.qp14_pairs[2 * k + 1]].push_back(q0 + d.qp14_pairs[2 * k]);
            for (int i = 0; i < N; ++i) {
                for (int q : q14[i]) qp14_q.push_back(q);
                qp14_first.push_back((int)qp14_q.size());
            }
        }
        // --- nbqq
        int off = 0;
        for (int s = 0; s < QG_MAXS; ++s) {
            T.qq0[s] = (int)qq_iq.size();
            int n = s < S ? d.nbqq_count[s] : 0;
            T.nqq[s] = n;
            for (int k = 0; k < n; ++k) {
                int p = off + k;
                qq_iq.push_back(q0 + d.nbqq_iq[p]);
                qq_j.push_back(atom0 + d.nbqq_j[p]);
                qq_jq.push_back(d.nbqq_jq[p] >= 0 ? q0 + d.nbqq_jq[p] : -1);
                qq_lj.push_back(d.nbqq_ljcod[p]);
                qq_els.push_back(d.nbqq_elscale[p]);
            }
            off += n;
            if (n) { qqblk_traj.push_back(t); qqblk_s.push_back(s); }
        }
        // --- Q bonded terms
        {
            int lib_b = (int)(qt_lib.size() / 4);
            for (int k = 0; k < d.nqbcod; ++k) for (int c = 0; c < 4; ++c) qt_lib.push_back(d.qbondlib[4 * k + c]);
            int lib_a = (int)(qt_lib.size() / 4);
            for (int k = 0; k < d.nqacod; ++k) for (int c = 0; c < 4; ++c) qt_lib.push_back(d.qanglib[4 * k + c]);
            int lib_t = (int)(qt_lib.size() / 4);
            for (int k = 0; k < d.nqtcod; ++k) { for (int c = 0; c < 3; ++c) qt_lib.push_back(d.qtorlib[3 * k + c]); qt_lib.push_back(0); }
            int lib_i = (int)(qt_lib.size() / 4);
            for (int k = 0; k < d.nqicod; ++k) { for (int c = 0; c < 2; ++c) qt_lib.push_back(d.qimplib[2 * k + c]); qt_lib.push_back(0); qt_lib.push_back(0); }
            auto addq = [&](const int32_t *rows, int nrow, int nat, int kind, int libo) {
                int w = nat + S;
                for (int r = 0; r < nrow; ++r) {
                    for (int a = 0; a < 4; ++a) qt_atoms.push_back(a < nat ? atom0 + rows[r * w + a] : atom0);
                    for (int s = 0; s < QG_MAXS; ++s) {
                        int c = s < S ? rows[r * w + nat + s] : 0;
                        qt_cod.push_back(c > 0 ? libo + c : 0);
                    }
                    qt_kind.push_back(kind); qt_traj.push_back(t);
                }
            };
            addq(d.qbnd, d.nqbond, 2, 0, lib_b);
            addq(d.qang, d.nqangle, 3, 1, lib_a);
            addq(d.qtor, d.nqtor, 4, 2, lib_t);
            addq(d.qimp, d.nqimp, 4, 3, lib_i);
        }
        // --- classical bonded terms, one padded segment per energy slot
        {
            int lb = (int)(bt_lib.size() / 4);
            for (int k = 0; k < d.nbndcod; ++k) { bt_lib.push_back(d.bondlib[2 * k]); bt_lib.push_back(d.bondlib[2 * k + 1]); bt_lib.push_back(0); bt_lib.push_back(0); }
            int la = (int)(bt_lib.size() / 4);
            for (int k = 0; k < d.nangcod; ++k) for (int c = 0; c < 4; ++c) bt_lib.push_back(d.anglib[4 * k + c]);
            int lt = (int)(bt_lib.size() / 4);
            for (int k = 0; k < d.ntorcod; ++k) for (int c = 0; c < 4; ++c) bt_lib.push_back((double)d.torlib[4 * k + c]);
            int li = (int)(bt_lib.size() / 4);
            for (int k = 0; k < d.nimpcod; ++k) { bt_lib.push_back((double)d.implib[2 * k]); bt_lib.push_back((double)d.implib[2 * k + 1]); bt_lib.push_back(0); bt_lib.push_back(0); }
            auto seg = [&](const int32_t *rows, int r0, int r1, int nat, int w, int kind, int libo, int slot) {
                if (r1 <= r0) return;
                size_t st = bt_cod.size();
                for (int r = r0; r < r1; ++r) {
                    for (int a = 0; a < 4; ++a) bt_atoms.push_back(a < nat ? atom0 + rows[r * w + a] : atom0);
                    bt_cod.push_back(libo + rows[r * w + nat] - 1);
                    bt_kind.push_back(kind);
                }
                while ((bt_cod.size() - st) % QG_BLOCK) {
                    for (int a = 0; a < 4; ++a) bt_atoms.push_back(0);
                    bt_cod.push_back(-1); bt_kind.push_back(0);
                }
                for (size_t b = st / QG_BLOCK; b < bt_cod.size() / QG_BLOCK; ++b) { bt_blk_traj.push_back(t); bt_blk_slot.push_back(slot); }
            };
            seg(d.bnd, 0, d.nbonds_solute, 2, 3, 0, lb, EA_P_BOND);
            seg(d.bnd, d.nbonds_solute, d.nbonds, 2, 3, 0, lb, EA_W_BOND);
            seg(d.ang, 0, d.nangles_solute, 3, 4, 1, la, EA_P_ANG);
            seg(d.ang, d.nangles_solute, d.nangles, 3, 4, 1, la, EA_W_ANG);
            seg(d.tor, 0, d.ntors_solute, 4, 5, 2, lt, EA_P_TOR);
            seg(d.tor, d.ntors_solute, d.ntors, 4, 5, 2, lt, EA_W_TOR);
            int ik = d.ff_type == 2 ? 4 : 3;
            seg(d.imp, 0, d.nimps_solute, 4, 5, ik, li, EA_P_IMP);
            seg(d.imp, d.nimps_solute, d.nimps, 4, 5, ik, li, EA_W_IMP);
        }
        // --- SHAKE
        T.shake_mol0 = (int)(shk_first.size() - 1);
        T.nshake_mol = d.shake_molecules;
        for (int m = 0; m < d.shake_molecules; ++m) {
            for (int c = d.shake_first[m]; c < d.shake_first[m + 1]; ++c) {
                shk_i.push_back(atom0 + d.shake_i[c]); shk_j.push_back(atom0 + d.shake_j[c]); shk_d2.push_back(d.shake_dist2[c]);
            }
            shk_first.push_back((int)shk_i.size());
            shk_traj.push_back(t);
        }
        if (d.shake_molecules) h->any_shake = 1;
        // --- off-diagonals
        std::vector<int> ost;
        for (int k = 0; k < d.noffd; ++k) {
            od_traj.push_back(t); od_ij.push_back(k); od_ij.push_back(0);
            od_kl.push_back(q0 + d.offd_kl[2 * k]); od_kl.push_back(q0 + d.offd_kl[2 * k + 1]);
            od_Amu.push_back(d.offd_Amu[2 * k]); od_Amu.push_back(d.offd_Amu[2 * k + 1]);
            ost.push_back(d.offd_ij[2 * k]); ost.push_back(d.offd_ij[2 * k + 1]);
        }
        h->offd_states.push_back(ost);
        h->info.push_back(T);
        h->nstates.push_back(S); h->natom.push_back(N); h->atom0.push_back(atom0);
        h->ncgp.push_back(d.ncgp); h->grp0.push_back(grp0); h->nqat.push_back(nq);
        h->nmol.push_back(0);
        h->max_natom = std::max(h->max_natom, N);
        atom0 += N; grp0 += d.ncgp; q0 += nq; type0 += nt; lj0 += nt * nt; qlib0 += nql; sc0 += nq * ntq * QG_MAXS;
    }
    // ---------------------------------------------------------- upload
    std::vector<void *> &A = h->allocs;
    DevSys &S = h->S;
    S.ntraj = ntraj; S.natom = atom0; S.ngrp = grp0; S.nq = q0;
    int gsz = 0;
    for (int t = 0; t < ntraj; ++t) gsz = std::max(gsz, h->ncgp[t]);
    S.nb_cap = 448;
    if (const char *e = getenv("QGPU_NB_CAP")) {   // list capacity per charge group (tests force overflow)
        int c = atoi(e);
        if (c > 0) S.nb_cap = c;
    }
    TrajInfo *ti; TrajState *ts;
    int rc;
    if ((rc = upload(A, h->info, &ti))) return rc;
    S.traj = ti;
    std::vector<TrajState> tsh(ntraj);
    for (auto &q : tsh) {
        q.Temp = q.Tfree = q.Ekin = 0.f; q.shake_iters = 0; q.shake_visits = 0;
        q.tsf_solute = q.tsf_solvent = 1.f; q.wshiftf = 0.f;
        q.Ekin_d = q.Temp_d = q.Tfree_d = 0.0; q.tsd_solute = q.tsd_solvent = 1.0;
        q.rnd = rnd0[&q - tsh.data()]; q.nh_s1 = q.nh_s2 = 1.0;
    }
    if ((rc = upload(A, tsh, &ts))) return rc;
    S.tstate = ts;
#define UP(vec, field)                                            \
    do {                                                          \
        decltype(vec.data()) p_;                                  \
        if ((rc = upload(A, vec, &p_))) return rc;                \
        S.field = p_;                                             \
    } while (0)
    UP(x, x); UP(v, v); UP(xtop, xtop); UP(winv, winv); UP(mass_atom, mass); UP(crg_d, crg_d);
    if ((rc = alloc0(A, (size_t)3 * atom0, &S.xx))) return rc;
    UP(pos, pos);
    if ((rc = alloc0(A, (size_t)atom0, &S.poslo))) return rc;
    if ((rc = alloc0(A, (size_t)atom0, &S.velf))) return rc;
    if ((rc = alloc0(A, (size_t)atom0, &S.wrec))) return rc;
    {
        // float copies for the per-step kernels; topology coordinates as hi/lo
        // offsets from each trajectory's origin
        std::vector<float> winvf(winv.begin(), winv.end()), massf(mass_atom.begin(), mass_atom.end());
        std::vector<float4> xth(atom0), xtl(atom0);
        for (int t = 0; t < ntraj; ++t)
            for (int i = h->atom0[t]; i < h->atom0[t] + h->natom[t]; ++i) {
                float r[3], e[3];
                for (int c = 0; c < 3; ++c) {
                    const double d = xtop[3 * (size_t)i + c] - h->info[t].origin[c];
                    r[c] = (float)d;
                    e[c] = (float)(d - (double)r[c]);
                }
                xth[i] = make_float4(r[0], r[1], r[2], 0.f);
                xtl[i] = make_float4(e[0], e[1], e[2], 0.f);
            }
        UP(winvf, winvf); UP(massf, massf); UP(xth, xtoph); UP(xtl, xtopl);
        std::vector<float2> d2hl(shk_d2.size());
        for (size_t c = 0; c < shk_d2.size(); ++c) {
            const float hi = (float)shk_d2[c];
            d2hl[c] = make_float2(hi, (float)(shk_d2[c] - (double)hi));
        }
        UP(d2hl, shk_d2hl);
        std::vector<float> qq_elsf(qq_els.begin(), qq_els.end()), qt_libf(qt_lib.begin(), qt_lib.end()),
            bt_libf(bt_lib.begin(), bt_lib.end());
        UP(qq_elsf, qq_elsf); UP(qt_libf, qt_libf); UP(bt_libf, bt_libf);
    }
    UP(atype, atype); UP(aq, aq); UP(aexcl, aexcl); UP(ashell, ashell); UP(atraj, atraj); UP(agrp, agrp);
    if ((rc = alloc0(A, (size_t)3 * atom0, &S.fx))) return rc;
    UP(exmask, exmask); UP(p14mask, p14mask); UP(exl_first, exlong_first); UP(exl_j, exlong_j); UP(exl_kind, exlong_kind);
    UP(avdw, avdw); UP(bvdw, bvdw); UP(avdw_d, avdw_d); UP(bvdw_d, bvdw_d); UP(ljcod, ljcod);
    UP(g_start, g_start); UP(g_atoms, g_atoms); UP(g_switch, g_switch); UP(g_kind, g_kind); UP(g_traj, g_traj);
    UP(g_excl, g_excl); UP(tile_g0, tile_g0); UP(tile_g1, tile_g1);
    if ((rc = alloc0(A, (size_t)3 * grp0, &S.g_cent))) return rc;
    if ((rc = alloc0(A, (size_t)grp0, &S.g_centf))) return rc;
    if ((rc = alloc0(A, (size_t)QG_NLRF * grp0, &S.g_phi))) return rc;
    if ((rc = alloc0(A, (size_t)QG_NPHI * grp0, &S.g_phif))) return rc;
    if ((rc = alloc0(A, (size_t)grp0, &S.nb_count))) return rc;
    if ((rc = alloc0(A, (size_t)grp0, &S.nb_nw))) return rc;
    if ((rc = alloc0(A, (size_t)scr_slots * QG_NLRF, &S.scr_phi))) return rc;
    if ((rc = alloc0(A, (size_t)scr_slots, &S.scr_cnt))) return rc;
    if ((rc = alloc0(A, (size_t)scr_slots * QG_CAPC, &S.scr_nb))) return rc;
    if ((rc = alloc0(A, (size_t)grp0 * S.nb_cap, &S.nb_list))) return rc;
    UP(q_atom, q_atom); UP(qcrg_f, qcrg_f); UP(qcrg_d, qcrg_d); UP(qiac, qiac);
    UP(qavdw, qavdw); UP(qbvdw, qbvdw); UP(qavdw_d, qavdw_d); UP(qbvdw_d, qbvdw_d); UP(sc_f, sc_f); UP(sc_d, sc_d);
    {
        float *p;
        if ((rc = upload(A, qw_A, &p))) return rc; S.qw_A = p;
        if ((rc = upload(A, qw_B, &p))) return rc; S.qw_B = p;
    }
    UP(qw_lj, qw_lj); UP(qw_sc, qw_sc); UP(qw_Ad, qw_Ad); UP(qw_Bd, qw_Bd);
    UP(qwh_A, qwh_A); UP(qwh_B, qwh_B); UP(qwh_Ad, qwh_Ad); UP(qwh_Bd, qwh_Bd);
    UP(ljA, ljA); UP(ljB, ljB); UP(ljA_d, ljA_d); UP(ljB_d, ljB_d);
    if ((rc = alloc0(A, (size_t)atom0, &S.qw_member))) return rc;
    if ((rc = alloc0(A, (size_t)atom0, &S.qp_member))) return rc;
    UP(xr_kind, xr_kind); UP(xr_at, xr_at); UP(xr_st, xr_st); UP(xr_blk_traj, xr_blk_traj);
    UP(xr_p, xr_p); UP(xr_pf, xr_pf);
    S.nxr = (int)xr_kind.size();
    {
        std::vector<int> gq(grp0, -1);
        UP(gq, g_qin);
        UP(mol_start, mol_start);
        UP(boxc0, boxc);
    }
    UP(qp_skip, qp_skip); UP(qp14_first, qp14_first); UP(qp14_q, qp14_q);
    UP(qq_iq, qq_iq); UP(qq_j, qq_j); UP(qq_jq, qq_jq); UP(qq_lj, qq_lj); UP(qq_els, qq_els);
    UP(qt_atoms, qt_atoms); UP(qt_cod, qt_cod); UP(qt_kind, qt_kind); UP(qt_traj, qt_traj); UP(qt_lib, qt_lib);
    S.nqt = (int)qt_kind.size();
    UP(bt_atoms, bt_atoms); UP(bt_cod, bt_cod); UP(bt_kind, bt_kind); UP(bt_lib, bt_lib);
    UP(bt_blk_traj, bt_blk_traj); UP(bt_blk_slot, bt_blk_slot);
    S.nbt = (int)bt_cod.size();
    UP(od_traj, od_traj); UP(od_ij, od_ij); UP(od_kl, od_kl); UP(od_Amu, od_Amu);
    S.nod = (int)od_traj.size();
    if ((rc = alloc0(A, (size_t)ntraj * QG_MAXOD * 2, &S.od_out))) return rc;
    UP(shk_first, shk_first); UP(shk_i, shk_i); UP(shk_j, shk_j); UP(shk_traj, shk_traj); UP(shk_d2, shk_d2);
    S.nshk_mol = (int)shk_traj.size();
    if ((rc = alloc0(A, (size_t)ntraj * QG_NE, &S.eacc))) return rc;
    UP(rs_i0, rs_i0); UP(rs_i1, rs_i1); UP(rs_ih, rs_ih); UP(rs_tc, rs_tc); UP(rs_traj, rs_traj); UP(rs_fk, rs_fk);
    S.nrs = (int)rs_i0.size();
    UP(aheavy, aheavy);
    UP(randva, randva); UP(lcg_a, lcg_a); UP(lcg_c, lcg_c);
    {
        std::vector<float> rvf(randva.begin(), randva.end());
        UP(rvf, randvaf);
    }
    if ((rc = alloc0(A, (size_t)ntraj * 2 * QG_MAXNH, &S.nh_state))) return rc;
    if ((rc = alloc0(A, (size_t)ntraj * QG_NFEP, &S.fep_acc))) return rc;
    if ((rc = alloc0(A, (size_t)ntraj, &S.fin_cnt))) return rc;
    h->ene_files.assign(ntraj, nullptr);
    if (!wp_state.empty()) { double *p_; if ((rc = upload(A, wp_state, &p_))) return rc; S.wp_state = p_; }
    for (char f : h->fused) h->can_fuse = h->can_fuse && f;
    h->all_fused = false;
    h->fused_d = h->can_fuse;
    h->ek_u0 = ek_u0; h->ek_un = ek_un; h->ek_a0 = ek_a0; h->ek_an = ek_an;
    {
        const size_t nblk_ek = std::max(uitem.size() / QG_BLOCK, uatom.size() / QG_UBLK) + 1;
        if ((rc = alloc0(A, (size_t)4 * nblk_ek, &S.ekin_part))) return rc;
        if ((rc = alloc0(A, (size_t)4 * nblk_ek, &S.ekin_fx))) return rc;
    }
    // the Ekin partials follow the update kernel in use
    set_ekin_layout(h);
    CK(cudaMemcpy((void *)S.traj, h->info.data(), h->info.size() * sizeof(TrajInfo), cudaMemcpyHostToDevice));
    if ((rc = alloc0(A, 2, &S.status))) return rc;   // [0] status bits, [1] 1 + trajectory of a SHAKE failure
    // block tables
    BlockTables &B = h->B;
    {
        int *p;
        if ((rc = upload(A, wgrp, &p))) return rc; B.wgrp = p; B.nwgrp = (int)wgrp.size();
        if ((rc = upload(A, satom, &p))) return rc; B.satom = p; B.nsatom = (int)satom.size();
        if ((rc = upload(A, scan_t0, &p))) return rc; B.scan_t0 = p;
        if ((rc = upload(A, scan_tn, &p))) return rc; B.scan_tn = p;
        if ((rc = upload(A, scan_traj, &p))) return rc; B.scan_traj = p; B.nscan = (int)scan_t0.size();
        if ((rc = upload(A, scan_chunk, &p))) return rc; B.scan_chunk = p;
        if ((rc = upload(A, uitem, &p))) return rc; B.uitem = p; B.nuitem = (int)uitem.size();
        if ((rc = upload(A, uatom, &p))) return rc; B.uatom = p; B.nuatom = (int)uatom.size();
        if ((rc = upload(A, ucon, &p))) return rc; B.ucon = p;
        uint8_t *pb;
        if ((rc = upload(A, ublk_water, &pb))) return rc; B.ublk_water = pb;
        if ((rc = upload(A, qqblk_traj, &p))) return rc; B.qqblk_traj = p;
        if ((rc = upload(A, qqblk_s, &p))) return rc; B.qqblk_s = p; B.nqqblk = (int)qqblk_traj.size();
        B.max_nqat = 0;
        for (int t = 0; t < ntraj; ++t) B.max_nqat = std::max(B.max_nqat, h->info[t].nqat);
        for (int t = 0; t < ntraj; ++t) B.any_atom |= h->info[t].any_atom;
        for (int t = 0; t < ntraj; ++t) B.pbc |= h->info[t].pbc;
        for (int t = 0; t < ntraj; ++t) B.hlj |= h->info[t].hlj;
        // any-atom lists in a box: the shift records of every neighbour entry
        bool anybox = false;
        for (int t = 0; t < ntraj; ++t) anybox |= h->info[t].any_atom && h->info[t].pbc;
        if (anybox) {
            if ((rc = alloc0(A, (size_t)S.ngrp * S.nb_cap, &S.nb_sha))) return rc;
            if ((rc = alloc0(A, (size_t)scr_slots * QG_CAPC, &S.scr_sha))) return rc;
        }
        B.npb = (int)pb_traj.size();
        B.nxrblk = (int)xr_blk_traj.size();
        // the whole batch
        B.g0 = 0; B.ng = S.ngrp; B.ublk0 = 0; B.qt0 = 0; B.nqt = S.nqt; B.od0 = 0; B.nod = S.nod;
        B.bt0 = 0; B.nbtblk = S.nbt / QG_BLOCK; B.rs0 = 0; B.nrs = S.nrs; B.xr0 = 0;
        // where each trajectory's part of every list starts (lists are in
        // trajectory order; padding entries carry -1 - trajectory)
        {
            auto first_at = [&](const std::vector<int> &tr, int t) {
                return (int)(std::lower_bound(tr.begin(), tr.end(), t) - tr.begin());
            };
            std::vector<int> tw, ts, tq;
            for (int e : wgrp) tw.push_back(e >= 0 ? g_traj[e] : -1 - e);
            for (int e : satom) ts.push_back(e >= 0 ? atraj[e] : -1 - e);
            h->lstart.resize(ntraj + 1);
            for (int t = 0; t <= ntraj; ++t) {
                qgpu_handle::ListStarts &L = h->lstart[t];
                L.wgrp = first_at(tw, t); L.satom = first_at(ts, t); L.scan = first_at(scan_traj, t);
                L.ublk = t < ntraj ? ek_a0[t] : (int)(uatom.size() / QG_UBLK);
                L.qqblk = first_at(qqblk_traj, t); L.wp = first_at(wp_traj, t); L.pb = first_at(pb_traj, t);
                L.bt = first_at(bt_blk_traj, t); L.qt = first_at(qt_traj, t); L.od = first_at(od_traj, t);
                L.rs = first_at(rs_traj, t); L.xr = first_at(xr_blk_traj, t);
                L.grp = t < ntraj ? h->info[t].grp0 : S.ngrp;
            }
        }
        if (B.npb) {
            int *p_;
            if ((rc = upload(A, pb_traj, &p_))) return rc; B.pb_traj = p_;
        }
        B.nwp = (int)wp_traj.size();
        if (B.nwp) {
            int *p_;
            if ((rc = upload(A, wp_traj, &p_))) return rc; B.wp_traj = p_;
            if ((rc = upload(A, wp_scr0, &p_))) return rc; B.wp_scr0 = p_;
            double *q_;
            if ((rc = alloc0(A, (size_t)wp_scr_n, &q_))) return rc; B.wp_scr = q_;
        }
    }
    if ((rc = alloc0(A, (size_t)ntraj * QG_REC, &h->ecur_d))) return rc;
    if ((rc = alloc0(A, 2, &h->zero_d))) return rc;
    if ((rc = alloc0(A, (size_t)3 * h->max_natom, &h->grad_d))) return rc;
    if ((rc = alloc0(A, 2, &h->recctl_d))) return rc;
    CK(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&h->ev_branch, cudaEventDisableTiming));
    make_branches(h, QG_DEFBRANCH);
    for (int g = 0; g < QG_MAXBRANCH; ++g) {
        CK(cudaStreamCreateWithFlags(&h->bstream[g], cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&h->bfork[g], cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&h->bdone[g], cudaEventDisableTiming));
        for (int k = 0; k < QG_NSIDE; ++k) {
            CK(cudaStreamCreateWithFlags(&h->bside[g][k], cudaStreamNonBlocking));
            CK(cudaEventCreateWithFlags(&h->bjoin[g][k], cudaEventDisableTiming));
        }
    }
    for (int k = 0; k < QG_NSIDE; ++k) {
        CK(cudaStreamCreateWithFlags(&h->side[k], cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&h->ev_join[k], cudaEventDisableTiming));
    }
    // float mirror of the starting coordinates
    LaunchCtx L{h->stream, &h->nlaunch};
    launch_mirror(S, B, L);
    CK(cudaStreamSynchronize(h->stream));
    CK(cudaGetLastError());
    return 0;
}

static int check_status(qgpu_handle *h) {
    int stw[2] = {0, 0};
    CK(cudaMemcpyAsync(stw, h->S.status, sizeof stw, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    CK(cudaGetLastError());
    const int st = stw[0];
    if (!st) return 0;
    const int zero[2] = {0, 0};
    CK(cudaMemcpy(h->S.status, zero, sizeof zero, cudaMemcpyHostToDevice));
    if (st & ST_LIST_OVERFLOW) return fail(QGPU_E_LIST_OVERFLOW, "neighbour list capacity %d exceeded", h->S.nb_cap);
    if (st & ST_SHAKE)
        return fail(QGPU_E_SHAKE, "shake failure: no convergence in 1000 iterations (trajectory %d)", stw[1] - 1);
    if (st & ST_NAN) return fail(QGPU_E_NAN, "a detected NaN in the temperature");
    if (st & ST_FIXED) return fail(QGPU_E_FIXED_RANGE, "force or energy outside the fixed-point range");
    return fail(QGPU_E_CUDA, "device status %d", st);
}

// Refreshes x/v from the float master after fused steps (API reads, list
// builds and FP64 evaluations read x/v).
static void ensure_double(qgpu_handle *h, LaunchCtx &L) {
    if (h->master == 1) launch_sync_double(h->S, h->B, L);
    h->master = 0;
}
static void after_steps(qgpu_handle *h) { h->master = h->all_fused ? 1 : 0; }

// temperature() before the first step (md_run, src/md.f90:6395-6398): the
// Ekin partials of the update layout in use
static void temperature_init(qgpu_handle *h, LaunchCtx &L) {
    if (h->all_fused) launch_update_f(h->S, h->B, L, EaccSel{EACC_FP32, h->zero_d, 0, 1}, h->NBcycle, 1);
    else if (h->fused_d) launch_update_d(h->S, h->B, L, EaccSel{EACC_FP32, h->zero_d, 0, 1}, 1);
    else { launch_update(h->S, h->B, L, 0); launch_wrec(h->S, h->B, L); }
}

// md: a list build of the MD loop, which first puts molecules back in the box
// (md_run :6483-6485); qgpu_build_lists alone is make_pair_lists.
static void list_ops(qgpu_handle *h, const BlockTables &B, LaunchCtx &L, bool md = true) {
    if (md) launch_put_back(h->S, B, L);
    launch_centers(h->S, B, L);
    launch_scan(h->S, B, L);
    launch_qmember(h->S, B, L, h->lists_built ? 0 : 1);
}
static void list_ops(qgpu_handle *h, LaunchCtx &L, bool md = true) { list_ops(h, h->B, L, md); }

// fp64_energy: every pair energy in FP64 (drop-in call); otherwise FP32 pair
// energies, with FP64 Q-atom energies on recorded steps (esel).
// The force kernels only read coordinates and tables and add into the
// fixed-point gradient and energy accumulators (integer adds, so the result
// does not depend on their order): they run concurrently on side streams that
// fork from and join back into the handle's stream (also inside graph
// capture).  The per-kernel profiler keeps them in one stream.
// The stream set a force stage forks onto: a fork event, side streams and
// their join events (the handle's own, or one branch's).
struct SideSet {
    cudaEvent_t fork;
    const cudaStream_t *side;
    const cudaEvent_t *join;
};
static void force_ops(qgpu_handle *h, const BlockTables &B, LaunchCtx &L, int terms, int emode, EaccSel esel,
                      SideSet ss) {
    const bool wpol = (terms & QGPU_TERMS_RESTRAINT) != 0;
    if (!(terms & QGPU_TERMS_NONBOND)) {
        launch_misc(h->S, B, L, terms, esel);
        if (wpol) launch_watpol(h->S, B, L, esel);
        return;
    }
    if (L.prof || !ss.fork) {
        launch_nb_water(h->S, B, L, 1, emode);
        launch_nb_solute(h->S, B, L, 1, emode);
        launch_qw(h->S, B, L, esel, emode);
        launch_qp(h->S, B, L, esel, emode);
        launch_misc(h->S, B, L, terms, esel);
        if (wpol) launch_watpol(h->S, B, L, esel);
        return;
    }
    cudaEventRecord(ss.fork, L.stream);
    LaunchCtx Ls[QG_NSIDE];
    for (int k = 0; k < QG_NSIDE; ++k) {
        cudaStreamWaitEvent(ss.side[k], ss.fork, 0);
        Ls[k] = LaunchCtx{ss.side[k], L.nlaunch};
    }
    launch_nb_water(h->S, B, L, 1, emode);
    launch_nb_solute(h->S, B, Ls[0], 1, emode);
    launch_qw(h->S, B, Ls[1], esel, emode);
    launch_qp(h->S, B, Ls[2], esel, emode);
    launch_misc(h->S, B, Ls[2], terms, esel);
    if (wpol) launch_watpol(h->S, B, Ls[1], esel);
    for (int k = 0; k < QG_NSIDE; ++k) {
        cudaEventRecord(ss.join[k], ss.side[k]);
        cudaStreamWaitEvent(L.stream, ss.join[k], 0);
    }
}
static void force_ops(qgpu_handle *h, LaunchCtx &L, int terms, int emode, EaccSel esel) {
    force_ops(h, h->B, L, terms, emode, esel, SideSet{h->ev_fork, h->side, h->ev_join});
}

static void step_ops(qgpu_handle *h, LaunchCtx &L, int k, int ene_every, int emode);
static void step_ops(qgpu_handle *h, const BlockTables &B, LaunchCtx &L, SideSet ss, int k, int ene_every, int emode);
// Pair-energy mode of an MD step: its pair energies are read only when the
// step is recorded (step % ene_every == 0).
static int step_emode(long long step, int ene_every) {
    return step % ene_every == 0 ? QG_PAIR_E_FP32 : QG_PAIR_E_NONE;
}

// One NBcycle block (list build + NBcycle steps + record-counter tick),
// captured once as a CUDA graph and replayed.
static int replay_block(qgpu_handle *h, LaunchCtx &L, int ene_every) {
    const int NB = h->NBcycle;
    if (h->graph && h->graph_ene_every != ene_every) { cudaGraphExecDestroy(h->graph); h->graph = nullptr; }
    if (!h->graph) {
        cudaGraph_t g;
        long long before = h->nlaunch;
        CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
        // a replayed block starts at a multiple of NB: where ene_every divides
        // NB the recorded steps of the block are fixed; where NB divides
        // ene_every only the block's first step can be recorded; elsewhere the
        // pair kernels keep their energies on every step
        auto emode_of = [&](int k) {
            int em = QG_PAIR_E_FP32;
            if (NB % ene_every == 0) em = step_emode(k, ene_every);
            else if (ene_every % NB == 0) em = k == 0 ? QG_PAIR_E_FP32 : QG_PAIR_E_NONE;
            return em;
        };
        if (h->nbranch > 1 && (h->all_fused || h->fused_d)) {
            // the trajectory groups are independent for the whole block: one
            // branch each (list build and NB steps), joined before the tick,
            // so that one group's FP64 update overlaps another's force kernels
            cudaEventRecord(h->ev_branch, h->stream);
            for (int g = 0; g < h->nbranch; ++g) {
                BlockTables &V = h->Bg[g];
                V.tune = h->B.tune;
                cudaStreamWaitEvent(h->bstream[g], h->ev_branch, 0);
                LaunchCtx Lg{h->bstream[g], L.nlaunch};
                const SideSet ss{h->bfork[g], h->bside[g], h->bjoin[g]};
                list_ops(h, V, Lg);
                for (int k = 0; k < NB; ++k) step_ops(h, V, Lg, ss, k, ene_every, emode_of(k));
                cudaEventRecord(h->bdone[g], h->bstream[g]);
                cudaStreamWaitEvent(h->stream, h->bdone[g], 0);
            }
        } else {
            list_ops(h, L);
            for (int k = 0; k < NB; ++k) step_ops(h, L, k, ene_every, emode_of(k));
        }
        launch_tick(L, h->recctl_d, NB);
        CK(cudaStreamEndCapture(h->stream, &g));
        CK(cudaGraphInstantiate(&h->graph, g, 0));
        cudaGraphDestroy(g);
        h->graph_nodes = h->nlaunch - before;
        h->graph_ene_every = ene_every;
        h->nlaunch = before;
    }
    CK(cudaGraphLaunch(h->graph, h->stream));
    h->nlaunch += h->graph_nodes;
    h->step += NB;
    return 0;
}

// one MD step of the trajectories of tables B on L's stream (fused forms);
// the separate-kernel forms always run the whole batch
static void step_ops(qgpu_handle *h, const BlockTables &B, LaunchCtx &L, SideSet ss, int k, int ene_every, int emode) {
    EaccSel esel{EACC_RECORD, h->recctl_d, k, ene_every};
    force_ops(h, B, L, QGPU_TERMS_ALL, emode, esel, ss);
    if (h->all_fused)
        launch_update_f(h->S, B, L, esel, h->NBcycle, 0, FIN_TEMP | FIN_STEP | FIN_NH, h->rec_d, h->rec_cap);
    else
        launch_update_d(h->S, B, L, esel, 0, FIN_TEMP | FIN_STEP | FIN_NH | FIN_EK64, h->rec_d, h->rec_cap);
}

static void step_ops(qgpu_handle *h, LaunchCtx &L, int k, int ene_every, int emode) {
    EaccSel esel{EACC_RECORD, h->recctl_d, k, ene_every};
    force_ops(h, L, QGPU_TERMS_ALL, emode, esel);
    if (h->all_fused) {
        // the update's last block per trajectory ends the step
        launch_update_f(h->S, h->B, L, esel, h->NBcycle, 0, FIN_TEMP | FIN_STEP | FIN_NH, h->rec_d, h->rec_cap);
    } else if (h->fused_d) {
        launch_update_d(h->S, h->B, L, esel, 0, FIN_TEMP | FIN_STEP | FIN_NH | FIN_EK64, h->rec_d, h->rec_cap);
    } else {
        launch_integrate(h->S, h->B, L);
        launch_shake(h->S, h->B, L, -1);
        launch_update(h->S, h->B, L, 2);
        launch_wrec(h->S, h->B, L);
        launch_finalize(h->S, L, FIN_TEMP | FIN_STEP | FIN_NH | FIN_EK64, h->rec_d, h->recctl_d, k, ene_every,
                        h->rec_cap);
    }
}

// ------------------------------------------------------------------ C-ABI
extern "C" {

int qgpu_last_error(char *buf, int32_t len) {
    if (!buf || len <= 0) return QGPU_E_INVALID;
    snprintf(buf, (size_t)len, "%s", g_err.c_str());
    return 0;
}

int qgpu_create(const qgpu_system_desc *descs, int32_t ntraj, qgpu_handle **out) {
    if (!descs || ntraj <= 0 || !out) return fail(QGPU_E_INVALID, "qgpu_create: bad arguments");
    // every descriptor is checked before any device call
    for (int t = 0; t < ntraj; ++t)
        if (int rc = validate(descs[t], t)) return rc;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(QGPU_E_CUDA, "no CUDA device");
    qgpu_handle *h = new qgpu_handle();
    int rc = create_impl(descs, ntraj, h);
    if (rc) { qgpu_destroy(h); *out = nullptr; return rc; }
    *out = h;
    return 0;
}

int qgpu_destroy(qgpu_handle *h) {
    if (!h) return 0;
    if (h->graph) cudaGraphExecDestroy(h->graph);
    if (h->stream) cudaStreamSynchronize(h->stream);
    for (void *p : h->allocs) cudaFree(p);
    if (h->rec_d) cudaFree(h->rec_d);
    for (int k = 0; k < QG_NSIDE; ++k) {
        if (h->side[k]) { cudaStreamSynchronize(h->side[k]); cudaStreamDestroy(h->side[k]); }
        if (h->ev_join[k]) cudaEventDestroy(h->ev_join[k]);
    }
    if (h->ev_fork) cudaEventDestroy(h->ev_fork);
    if (h->ev_branch) cudaEventDestroy(h->ev_branch);
    for (int g = 0; g < QG_MAXBRANCH; ++g) {
        if (h->bstream[g]) { cudaStreamSynchronize(h->bstream[g]); cudaStreamDestroy(h->bstream[g]); }
        if (h->bfork[g]) cudaEventDestroy(h->bfork[g]);
        if (h->bdone[g]) cudaEventDestroy(h->bdone[g]);
        for (int k = 0; k < QG_NSIDE; ++k) {
            if (h->bside[g][k]) { cudaStreamSynchronize(h->bside[g][k]); cudaStreamDestroy(h->bside[g][k]); }
            if (h->bjoin[g][k]) cudaEventDestroy(h->bjoin[g][k]);
        }
    }
    for (FILE *f : h->ene_files)
        if (f) fclose(f);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return 0;
}

int qgpu_ntraj(const qgpu_handle *h) { return h ? h->ntraj : 0; }

int64_t qgpu_kernel_launches(const qgpu_handle *h) { return h ? h->nlaunch : 0; }

int qgpu_set_coords(qgpu_handle *h, int32_t traj, const double *x, const double *v) {
    if (!h || traj < 0 || traj >= h->ntraj) return fail(QGPU_E_INVALID, "bad trajectory index");
    size_t off = 3 * (size_t)h->atom0[traj], n = 3 * (size_t)h->natom[traj];
    LaunchCtx L{h->stream, &h->nlaunch};
    ensure_double(h, L);
    if (x) CK(cudaMemcpyAsync(h->S.x + off, x, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    if (v) CK(cudaMemcpyAsync(h->S.v + off, v, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    launch_mirror_range(h->S, L, h->atom0[traj], h->natom[traj]);
    CK(cudaStreamSynchronize(h->stream));
    return 0;
}

int qgpu_set_coords_all(qgpu_handle *h, const double *x, const double *v) {
    if (!h) return fail(QGPU_E_INVALID, "null handle");
    const size_t n = 3 * (size_t)h->S.natom;
    LaunchCtx L{h->stream, &h->nlaunch};
    // x and v both replaced: nothing of the float master needs keeping
    if (x && v) h->master = 0;
    else ensure_double(h, L);
    if (x) CK(cudaMemcpyAsync(h->S.x, x, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    if (v) CK(cudaMemcpyAsync(h->S.v, v, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    launch_mirror_range(h->S, L, 0, h->S.natom);
    CK(cudaStreamSynchronize(h->stream));
    return 0;
}

int qgpu_get_coords_all(qgpu_handle *h, double *x, double *v) {
    if (!h) return fail(QGPU_E_INVALID, "null handle");
    const size_t n = 3 * (size_t)h->S.natom;
    LaunchCtx L{h->stream, &h->nlaunch};
    ensure_double(h, L);
    if (x) CK(cudaMemcpyAsync(x, h->S.x, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    if (v) CK(cudaMemcpyAsync(v, h->S.v, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return 0;
}

int qgpu_get_coords(qgpu_handle *h, int32_t traj, double *x, double *v) {
    if (!h || traj < 0 || traj >= h->ntraj) return fail(QGPU_E_INVALID, "bad trajectory index");
    size_t off = 3 * (size_t)h->atom0[traj], n = 3 * (size_t)h->natom[traj];
    LaunchCtx L{h->stream, &h->nlaunch};
    ensure_double(h, L);
    if (x) CK(cudaMemcpyAsync(x, h->S.x + off, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    if (v) CK(cudaMemcpyAsync(v, h->S.v + off, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return 0;
}

int qgpu_build_lists(qgpu_handle *h) {
    if (!h) return fail(QGPU_E_INVALID, "null handle");
    LaunchCtx L{h->stream, &h->nlaunch};
    ensure_double(h, L);
    list_ops(h, L, false);
    h->lists_built = 1;
    return check_status(h);
}

static void unpack_row(const double *R, int S, qgpu_energies *E, qgpu_qenergy *EQ) {
    if (E) memcpy(E, R + QG_REC_E, sizeof(qgpu_energies));
    if (EQ)
        for (int s = 0; s < S; ++s) memcpy(&EQ[s], R + QG_REC_EQ + 15 * s, sizeof(qgpu_qenergy));
}

int qgpu_forces(qgpu_handle *h, int32_t traj, int32_t terms, double *d, qgpu_energies *E, qgpu_qenergy *EQ) {
    if (!h || traj < 0 || traj >= h->ntraj) return fail(QGPU_E_INVALID, "bad trajectory index");
    if (!h->lists_built) return fail(QGPU_E_INVALID, "qgpu_forces before qgpu_build_lists");
    LaunchCtx L{h->stream, &h->nlaunch};
    ensure_double(h, L);
    CK(cudaMemsetAsync(h->S.fx, 0, 3 * (size_t)h->S.natom * sizeof(unsigned long long), h->stream));
    if (terms & QGPU_TERMS_STEP_PRECISION)
        force_ops(h, L, terms, QG_PAIR_E_FP32, EaccSel{EACC_FP32, h->recctl_d, 0, 1});
    else
        force_ops(h, L, terms, QG_PAIR_E_FP64, EaccSel{EACC_FP64, h->recctl_d, 0, 1});
    launch_finalize(h->S, L, 0, h->ecur_d, h->zero_d, 0, 1, 1);
    std::vector<double> row(QG_REC);
    CK(cudaMemcpyAsync(row.data(), h->ecur_d + (size_t)traj * QG_REC, QG_REC * sizeof(double), cudaMemcpyDeviceToHost,
                       h->stream));
    if (d) {
        launch_grad_to_double(h->S, L, h->grad_d, h->atom0[traj], h->natom[traj]);
        CK(cudaMemcpyAsync(d, h->grad_d, 3 * (size_t)h->natom[traj] * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    }
    if (int rc = check_status(h)) return rc;
    unpack_row(row.data(), h->nstates[traj], E, EQ);
    return 0;
}

int qgpu_shake(qgpu_handle *h, int32_t traj, const double *xx, double *x, int32_t *niter) {
    if (!h || traj < 0 || traj >= h->ntraj || !xx || !x) return fail(QGPU_E_INVALID, "bad arguments");
    size_t off = 3 * (size_t)h->atom0[traj], n = 3 * (size_t)h->natom[traj];
    LaunchCtx L{h->stream, &h->nlaunch};
    ensure_double(h, L);
    CK(cudaMemcpyAsync(h->S.xx + off, xx, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->S.x + off, x, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemsetAsync(&h->S.tstate[traj].shake_iters, 0, sizeof(int), h->stream));
    launch_shake(h->S, h->B, L, traj);
    launch_mirror(h->S, h->B, L);
    CK(cudaMemcpyAsync(x, h->S.x + off, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    int it = 0;
    CK(cudaMemcpyAsync(&it, &h->S.tstate[traj].shake_iters, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    if (int rc = check_status(h)) return rc;
    if (niter) *niter = h->info[traj].nshake_mol ? it / h->info[traj].nshake_mol : 0;
    return 0;
}

int qgpu_shake_counts(qgpu_handle *h, int64_t *sweeps, int64_t *visits) {
    if (!h) return fail(QGPU_E_INVALID, "null handle");
    std::vector<TrajState> ts(h->ntraj);
    CK(cudaStreamSynchronize(h->stream));
    CK(cudaMemcpy(ts.data(), h->S.tstate, ts.size() * sizeof(TrajState), cudaMemcpyDeviceToHost));
    int64_t sw = 0, vi = 0;
    for (const TrajState &q : ts) { sw += (unsigned)q.shake_iters; vi += (unsigned)q.shake_visits; }
    for (int t = 0; t < h->ntraj; ++t) {
        CK(cudaMemset(&h->S.tstate[t].shake_iters, 0, sizeof(int)));
        CK(cudaMemset(&h->S.tstate[t].shake_visits, 0, sizeof(int)));
    }
    if (sweeps) *sweeps = sw;
    if (visits) *visits = vi;
    return 0;
}

int qgpu_get_temperature(qgpu_handle *h, int32_t traj, double *out4) {
    if (!h || traj < 0 || traj >= h->ntraj || !out4) return fail(QGPU_E_INVALID, "bad arguments");
    TrajState ts;
    CK(cudaMemcpyAsync(&ts, h->S.tstate + traj, sizeof ts, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    out4[0] = ts.Temp_d; out4[1] = ts.Tfree_d; out4[2] = ts.tsd_solute; out4[3] = ts.tsd_solvent;
    return 0;
}

int qgpu_get_group_pairs(qgpu_handle *h, int32_t traj, int32_t *pairs, int64_t cap, int64_t *npairs) {
    if (!h || traj < 0 || traj >= h->ntraj) return fail(QGPU_E_INVALID, "bad trajectory index");
    int G = h->ncgp[traj], g0 = h->grp0[traj], C = h->S.nb_cap;
    int N = h->natom[traj], a0 = h->atom0[traj];
    std::vector<int> cnt(G), nw(G), lst((size_t)G * C), agrp(N);
    CK(cudaMemcpy(cnt.data(), h->S.nb_count + g0, G * sizeof(int), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(nw.data(), h->S.nb_nw + g0, G * sizeof(int), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(lst.data(), h->S.nb_list + (size_t)g0 * C, (size_t)G * C * sizeof(int), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(agrp.data(), h->S.agrp + a0, N * sizeof(int), cudaMemcpyDeviceToHost));
    int64_t n = 0;
    for (int g = 0; g < G; ++g)
        for (int k = 0; k < cnt[g]; ++k) {
            int e = lst[(size_t)g * C + k];
            int o = (k < nw[g] ? agrp[e - a0] : e) - g0;   // water entries hold the O atom
            if (o > g) {
                if (pairs && n < cap) { pairs[2 * n] = g; pairs[2 * n + 1] = o; }
                n++;
            }
        }
    if (npairs) *npairs = n;
    return 0;
}

int qgpu_get_q_lists(qgpu_handle *h, int32_t traj, int32_t *qp_atoms, int64_t cap_qp, int64_t *nqp,
                     int32_t *qw_waters, int64_t cap_qw, int64_t *nqw) {
    if (!h || traj < 0 || traj >= h->ntraj) return fail(QGPU_E_INVALID, "bad trajectory index");
    const int N = h->natom[traj], a0 = h->atom0[traj];
    std::vector<uint8_t> qp(N), qw(N);
    CK(cudaStreamSynchronize(h->stream));
    CK(cudaMemcpy(qp.data(), h->S.qp_member + a0, N, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(qw.data(), h->S.qw_member + a0, N, cudaMemcpyDeviceToHost));
    const int nsol = h->info[traj].nat_solute;
    int64_t np = 0, nw = 0;
    for (int i = 0; i < N; ++i) {
        if (i < nsol && qp[i]) {
            if (qp_atoms && np < cap_qp) qp_atoms[np] = i;
            np++;
        }
        // water O atoms: the first atom of each 3-atom solvent molecule
        if (i >= nsol && (i - nsol) % 3 == 0 && qw[i]) {
            if (qw_waters && nw < cap_qw) qw_waters[nw] = i;
            nw++;
        }
    }
    if (nqp) *nqp = np;
    if (nqw) *nqw = nw;
    return 0;
}

int qgpu_get_lrf(qgpu_handle *h, int32_t traj, double *lrf43) {
    if (!h || traj < 0 || traj >= h->ntraj || !lrf43) return fail(QGPU_E_INVALID, "bad arguments");
    int G = h->ncgp[traj], g0 = h->grp0[traj];
    std::vector<double> c(3 * (size_t)G), a((size_t)QG_NLRF * G);
    std::vector<float> af((size_t)QG_NLRF * G);
    CK(cudaMemcpy(c.data(), h->S.g_cent + 3 * (size_t)g0, c.size() * sizeof(double), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(af.data(), h->S.g_phi + (size_t)QG_NLRF * g0, af.size() * sizeof(float), cudaMemcpyDeviceToHost));
    for (size_t k = 0; k < af.size(); ++k) a[k] = af[k];
    // symmetric sums -> the 3 + 1 + 3 + 9 + 27 layout of LRF_TYPE (src/md.f90:444-450)
    static const int p2[3][3] = {{8, 11, 12}, {11, 9, 13}, {12, 13, 10}};
    for (int g = 0; g < G; ++g) {
        const double *A = a.data() + (size_t)QG_NLRF * g;
        double *o = lrf43 + 43 * (size_t)g;
        for (int k = 0; k < 3; ++k) o[k] = c[3 * g + k];
        o[3] = A[0];
        for (int k = 0; k < 3; ++k) o[4 + k] = -A[2 + k];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) o[7 + 3 * i + j] = A[p2[i][j]] - (i == j ? A[1] : 0.0);
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j)
                for (int k = 0; k < 3; ++k) {
                    int s[3] = {i, j, k};
                    std::sort(s, s + 3);
                    int idx;
                    if (s[0] == s[2]) idx = 14 + s[0];                       // xxx yyy zzz
                    else if (s[0] == 0 && s[1] == 0) idx = s[2] == 1 ? 17 : 18; // xxy xxz
                    else if (s[0] == 0 && s[1] == 1 && s[2] == 1) idx = 19;    // xyy
                    else if (s[0] == 0 && s[1] == 2) idx = 20;                 // xzz
                    else if (s[0] == 1 && s[1] == 1) idx = 21;                 // yyz
                    else if (s[0] == 1 && s[1] == 2) idx = 22;                 // yzz
                    else idx = 23;                                             // xyz
                    double val = 5.0 * A[idx];
                    if (i == j) val += A[5 + k];
                    if (i == k) val += A[5 + j];
                    if (j == k) val += A[5 + i];
                    o[16 + 9 * i + 3 * j + k] = val;
                }
    }
    return 0;
}

void *qgpu_stream(qgpu_handle *h) { return h ? (void *)h->stream : nullptr; }

// Runs nsteps MD steps launch by launch (no graph) with CUDA events around
// every kernel and returns, per kernel name, total milliseconds and launches.
int qgpu_profile(qgpu_handle *h, int32_t nsteps, char *names, double *ms, int64_t *counts, int32_t cap,
                 int32_t *nkernels) {
    if (!h || nsteps <= 0) return fail(QGPU_E_INVALID, "bad arguments");
    KernelProfiler P;
    LaunchCtx L{h->stream, &h->nlaunch, &P};
    if (!h->rec_d) {
        CK(cudaMalloc(&h->rec_d, (size_t)256 * h->ntraj * QG_REC * sizeof(double)));
        h->rec_cap = 256;
    }
    const int ene_every = 1 << 30;
    int ctl[2] = {(int)h->step, (int)((h->step + ene_every - 1) / ene_every)};
    launch_set_ctl(L, h->recctl_d, 2, ctl[0], ctl[1]);
    ensure_double(h, L);
    for (int k = 0; k < nsteps; ++k) {
        if (h->step % h->NBcycle == 0) { list_ops(h, L); h->lists_built = 1; }
        step_ops(h, L, 0, ene_every, step_emode(h->step, ene_every));
        launch_tick(L, h->recctl_d, 1);
        h->step += 1;
    }
    after_steps(h);
    CK(cudaStreamSynchronize(h->stream));
    std::map<std::string, std::pair<double, long long>> acc;
    for (auto &r : P.recs) {
        float t = 0;
        CK(cudaEventElapsedTime(&t, r.a, r.b));
        auto &a = acc[r.name];
        a.first += t; a.second += 1;
        cudaEventDestroy(r.a); cudaEventDestroy(r.b);
    }
    int n = 0;
    for (auto &kv : acc) {
        if (n < cap) {
            if (names) snprintf(names + 64 * n, 64, "%s", kv.first.c_str());
            if (ms) ms[n] = kv.second.first;
            if (counts) counts[n] = kv.second.second;
        }
        n++;
    }
    if (nkernels) *nkernels = n;
    return check_status(h);
}

// Enqueues nsteps of device work (graph replays where a whole NBcycle block
// fits) without waiting; energies of every ene_every-th step go to the device
// record buffer.  Errors surface at the next qgpu_sync / qgpu_run.
int qgpu_enqueue(qgpu_handle *h, int32_t nsteps, int32_t ene_every) {
    if (!h || nsteps < 0) return fail(QGPU_E_INVALID, "bad arguments");
    if (ene_every <= 0) ene_every = 1 << 30;
    if (h->graph && h->graph_ene_every != ene_every) { cudaGraphExecDestroy(h->graph); h->graph = nullptr; }
    LaunchCtx L{h->stream, &h->nlaunch};
    if (!h->rec_d) {
        CK(cudaMalloc(&h->rec_d, (size_t)256 * h->ntraj * QG_REC * sizeof(double)));
        h->rec_cap = 256;
    }
    ensure_double(h, L);
    if (!h->temp_init) {
        CK(cudaMemsetAsync(h->S.fx, 0, 3 * (size_t)h->S.natom * sizeof(unsigned long long), h->stream));
        CK(cudaMemsetAsync(h->S.eacc, 0, (size_t)h->ntraj * QG_NE * sizeof(unsigned long long), h->stream));
        temperature_init(h, L);
        launch_finalize(h->S, L, FIN_TEMP | (h->nh_ready ? 0 : FIN_NH) | (h->all_fused ? 0 : FIN_EK64), nullptr,
                        h->zero_d, 0, 1, 0);
        h->nh_ready = 1;
        h->temp_init = 1;
    }
    int ctl[2] = {(int)h->step, (int)((h->step + ene_every - 1) / ene_every)};
    launch_set_ctl(L, h->recctl_d, 2, ctl[0], ctl[1]);
    const int NB = h->NBcycle;
    const long long end = h->step + nsteps;
    while (h->step < end) {
        if (h->step % NB == 0 && end - h->step >= NB && h->lists_built) {
            if (int rc = replay_block(h, L, ene_every)) return rc;
        } else {
            if (h->step % NB == 0) { list_ops(h, L); h->lists_built = 1; }
            step_ops(h, L, 0, ene_every, step_emode(h->step, ene_every));
            launch_tick(L, h->recctl_d, 1);
            h->step += 1;
        }
    }
    after_steps(h);
    return 0;
}

int qgpu_sync(qgpu_handle *h) {
    if (!h) return fail(QGPU_E_INVALID, "null handle");
    return check_status(h);
}

// ------------------------------------------------------------ autotuner
// Chooses the launch shapes of the pair kernels by timing every variant on
// this handle's own lists (CUDA events on the handle's stream, median of 7
// launches after 2 warm-up launches).  The choice is kept per device and
// system size for the later handles of the process.
static std::map<std::string, Tuning> g_tune_cache;

static std::string tune_key(const qgpu_handle *h) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceProp p{};
    cudaGetDeviceProperties(&p, dev);
    char buf[256];
    snprintf(buf, sizeof buf, "%s/%d/%d/%d/%d/%d", p.name, p.multiProcessorCount, h->ntraj, h->S.natom, h->B.nwgrp,
             h->B.nsatom);
    return buf;
}

static int time_variant(qgpu_handle *h, LaunchCtx &L, void (*launch)(qgpu_handle *, LaunchCtx &), float *ms) {
    cudaEvent_t a, b;
    CK(cudaEventCreate(&a));
    CK(cudaEventCreate(&b));
    for (int w = 0; w < 2; ++w) launch(h, L);
    std::vector<float> t;
    for (int r = 0; r < 7; ++r) {
        CK(cudaEventRecord(a, h->stream));
        launch(h, L);
        CK(cudaEventRecord(b, h->stream));
        CK(cudaEventSynchronize(b));
        float x = 0.f;
        CK(cudaEventElapsedTime(&x, a, b));
        t.push_back(x);
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    std::sort(t.begin(), t.end());
    *ms = t[t.size() / 2];
    return 0;
}

// the shapes are timed in the form most MD steps run (no pair energies)
static void tune_water(qgpu_handle *h, LaunchCtx &L) { launch_nb_water(h->S, h->B, L, 1, QG_PAIR_E_NONE); }
static void tune_solute(qgpu_handle *h, LaunchCtx &L) { launch_nb_solute(h->S, h->B, L, 1, QG_PAIR_E_NONE); }
// the whole force stage of an unrecorded MD step, its kernels concurrent on
// the side streams as in the step itself
static void tune_forces(qgpu_handle *h, LaunchCtx &L) {
    force_ops(h, L, QGPU_TERMS_ALL, QG_PAIR_E_NONE, EaccSel{EACC_RECORD, h->zero_d, 0, 0});
}
static void tune_qw(qgpu_handle *h, LaunchCtx &L) {
    launch_qw(h->S, h->B, L, EaccSel{EACC_FP32, h->zero_d, 0, 1}, QG_PAIR_E_NONE);
}

int qgpu_set_tuning(qgpu_handle *h, const int32_t *tuning) {
    if (!h || !tuning) return fail(QGPU_E_INVALID, "qgpu_set_tuning: bad arguments");
    const int lw = tuning[0], mb = tuning[1], ls = tuning[2], lq = tuning[3], uw = tuning[4];
    if ((lw != 4 && lw != 8 && lw != 16) || (mb != 1 && mb != 6) || (ls != 4 && ls != 8 && ls != 16) ||
        (lq != 0 && lq != 1 && lq != 2 && lq != 4) || (uw != 1 && uw != 2 && uw != 3 && uw != 4))
        return fail(QGPU_E_INVALID, "qgpu_set_tuning: unsupported shape");
    CK(cudaStreamSynchronize(h->stream));
    h->B.tune.lw_water = lw; h->B.tune.minb_water = mb; h->B.tune.lw_solute = ls; h->B.tune.lg_qw = lq;
    h->B.tune.unroll_water = uw;
    if (h->graph) { cudaGraphExecDestroy(h->graph); h->graph = nullptr; }
    return 0;
}

int qgpu_autotune(qgpu_handle *h, int32_t *tuning) {
    if (!h) return fail(QGPU_E_INVALID, "null handle");
    const std::string key = tune_key(h);
    auto it = g_tune_cache.find(key);
    if (it == g_tune_cache.end()) {
        if (!h->lists_built)
            if (int rc = qgpu_build_lists(h)) return rc;
        LaunchCtx L{h->stream, &h->nlaunch};
        ensure_double(h, L);
        CK(cudaStreamSynchronize(h->stream));
        Tuning best = h->B.tune;
        float t, tb = 1e30f;
        if (h->B.nwgrp) {
            for (int lw : {4, 8, 16})
                for (int mb : {1, 6})
                    for (int uw : {1, 2, 3, 4}) {
                        h->B.tune.lw_water = lw; h->B.tune.minb_water = mb; h->B.tune.unroll_water = uw;
                        if (int rc = time_variant(h, L, tune_water, &t)) return rc;
                        if (t < tb) { tb = t; best.lw_water = lw; best.minb_water = mb; best.unroll_water = uw; }
                    }
            h->B.tune.lw_water = best.lw_water; h->B.tune.minb_water = best.minb_water;
            h->B.tune.unroll_water = best.unroll_water;
            tb = 1e30f;
            for (int lq : {1, 2, 4}) {
                h->B.tune.lg_qw = lq;
                if (int rc = time_variant(h, L, tune_qw, &t)) return rc;
                if (t < tb) { tb = t; best.lg_qw = lq; }
            }
            h->B.tune.lg_qw = best.lg_qw;
        }
        if (h->B.nsatom) {
            tb = 1e30f;
            for (int ls : {4, 8, 16}) {
                h->B.tune.lw_solute = ls;
                if (int rc = time_variant(h, L, tune_solute, &t)) return rc;
                if (t < tb) { tb = t; best.lw_solute = ls; }
            }
        }
        h->B.tune = best;
        // Second pass: in a step the force kernels share the GPU (side
        // streams), and the shape that is fastest alone is not always the
        // one that overlaps best.  Coordinate descent from the first pass's
        // choice on the time of the concurrent force stage.
        if (h->B.nwgrp && h->ev_fork) {
            tb = 1e30f;
            for (int lw : {4, 8, 16})
                for (int mb : {1, 6})
                    for (int uw : {1, 2, 3, 4}) {
                        h->B.tune.lw_water = lw; h->B.tune.minb_water = mb; h->B.tune.unroll_water = uw;
                        if (int rc = time_variant(h, L, tune_forces, &t)) return rc;
                        if (t < tb) { tb = t; best.lw_water = lw; best.minb_water = mb; best.unroll_water = uw; }
                    }
            h->B.tune = best;
            if (h->B.nsatom) {
                tb = 1e30f;
                for (int ls : {4, 8, 16}) {
                    h->B.tune.lw_solute = ls;
                    if (int rc = time_variant(h, L, tune_forces, &t)) return rc;
                    if (t < tb) { tb = t; best.lw_solute = ls; }
                }
                h->B.tune = best;
            }
            tb = 1e30f;
            for (int lq : {1, 2, 4}) {
                h->B.tune.lg_qw = lq;
                if (int rc = time_variant(h, L, tune_forces, &t)) return rc;
                if (t < tb) { tb = t; best.lg_qw = lq; }
            }
            h->B.tune = best;
        }
        // the timing launches added into the gradient and energies
        CK(cudaMemsetAsync(h->S.fx, 0, 3 * (size_t)h->S.natom * sizeof(unsigned long long), h->stream));
        CK(cudaMemsetAsync(h->S.eacc, 0, (size_t)h->ntraj * QG_NE * sizeof(unsigned long long), h->stream));
        CK(cudaStreamSynchronize(h->stream));
        if (int rc = check_status(h)) return rc;
        g_tune_cache[key] = best;
    } else {
        h->B.tune = it->second;
    }
    if (h->graph) { cudaGraphExecDestroy(h->graph); h->graph = nullptr; }
    if (tuning) {
        tuning[0] = h->B.tune.lw_water; tuning[1] = h->B.tune.minb_water;
        tuning[2] = h->B.tune.lw_solute; tuning[3] = h->B.tune.lg_qw; tuning[4] = h->B.tune.unroll_water;
    }
    return 0;
}

int qgpu_set_step(qgpu_handle *h, int64_t istep) {
    if (!h || istep < 0 || istep > 2000000000LL) return fail(QGPU_E_INVALID, "qgpu_set_step: bad arguments");
    h->step = istep;
    LaunchCtx L{h->stream, &h->nlaunch};
    launch_set_ctl(L, h->recctl_d, 1, (int)istep);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(h->stream));
    return 0;
}

int qgpu_set_branches(qgpu_handle *h, int32_t n) {
    if (!h || n < 1 || n > QG_MAXBRANCH) return fail(QGPU_E_INVALID, "qgpu_set_branches: n must be 1..%d", QG_MAXBRANCH);
    CK(cudaStreamSynchronize(h->stream));
    make_branches(h, n);
    if (h->graph) { cudaGraphExecDestroy(h->graph); h->graph = nullptr; }
    return 0;
}

int qgpu_get_branches(const qgpu_handle *h) { return h ? h->nbranch : 0; }

int qgpu_set_precision(qgpu_handle *h, int32_t mode) {
    if (!h || (mode != QGPU_PRECISION_MIXED && mode != QGPU_PRECISION_FP64 && mode != QGPU_PRECISION_FP64_UNFUSED))
        return fail(QGPU_E_INVALID, "qgpu_set_precision: bad arguments");
    const bool fused_f = mode == QGPU_PRECISION_MIXED && h->can_fuse;
    const bool fused_d = mode == QGPU_PRECISION_FP64 && h->can_fuse;
    if (fused_f == h->all_fused && fused_d == h->fused_d) return 0;
    LaunchCtx L{h->stream, &h->nlaunch};
    ensure_double(h, L);          // x/v from the float master before leaving it
    // entering the float master: its velocities (and hi/lo positions) from x/v
    if (fused_f) launch_mirror(h->S, h->B, L);
    CK(cudaStreamSynchronize(h->stream));
    h->all_fused = fused_f;
    h->fused_d = fused_d;
    set_ekin_layout(h);
    CK(cudaMemcpy((void *)h->S.traj, h->info.data(), h->info.size() * sizeof(TrajInfo), cudaMemcpyHostToDevice));
    if (h->graph) { cudaGraphExecDestroy(h->graph); h->graph = nullptr; }
    // the Ekin partials of the new layout are formed again before the next step
    h->temp_init = 0;
    return 0;
}

int qgpu_ene_open(qgpu_handle *h, int32_t traj, const char *path) {
    if (!h || traj < 0 || traj >= h->ntraj || !path) return fail(QGPU_E_INVALID, "qgpu_ene_open: bad arguments");
    if (h->ene_files[traj]) fclose(h->ene_files[traj]);
    h->ene_files[traj] = fopen(path, "wb");
    if (!h->ene_files[traj]) return fail(QGPU_E_INVALID, "qgpu_ene_open: cannot open %s", path);
    if (qgpu_ene_write_header(h->ene_files[traj], "5.06 (qsource_gb300)"))
        return fail(QGPU_E_INVALID, "qgpu_ene_open: cannot write %s", path);
    return 0;
}

int qgpu_ene_close(qgpu_handle *h, int32_t traj) {
    if (!h || traj < 0 || traj >= h->ntraj) return fail(QGPU_E_INVALID, "qgpu_ene_close: bad arguments");
    if (h->ene_files[traj] && fclose(h->ene_files[traj]) != 0) {
        h->ene_files[traj] = nullptr;
        return fail(QGPU_E_INVALID, "qgpu_ene_close: write failed");
    }
    h->ene_files[traj] = nullptr;
    return 0;
}

int qgpu_fep_start(qgpu_handle *h, int32_t nwin, const int32_t *chain, double kT, int32_t nskip) {
    if (!h || nwin < 2 || !chain || !(kT > 0) || nskip < 0) return fail(QGPU_E_INVALID, "qgpu_fep_start: bad arguments");
    std::vector<char> seen(h->ntraj, 0);
    for (int w = 0; w < nwin; ++w) {
        const int t = chain[w];
        if (t < 0 || t >= h->ntraj || seen[t]) return fail(QGPU_E_INVALID, "qgpu_fep_start: bad chain entry %d", w);
        if (h->nstates[t] != h->nstates[chain[0]])
            return fail(QGPU_E_INVALID, "qgpu_fep_start: windows with different state counts");
        seen[t] = 1;
    }
    LaunchCtx L{h->stream, &h->nlaunch};
    CK(cudaStreamSynchronize(h->stream));
    for (int t = 0; t < h->ntraj; ++t) h->info[t].fep_on = 0;
    for (int w = 0; w < nwin; ++w) {
        TrajInfo &T = h->info[chain[w]];
        T.fep_on = 1; T.fep_kT = kT; T.fep_nskip = nskip;
        T.fep_has_f = w + 1 < nwin; T.fep_has_r = w > 0;
        for (int s = 0; s < QG_MAXS; ++s) {
            T.fep_lamf[s] = T.fep_has_f ? h->info[chain[w + 1]].lambda[s] : 0.0;
            T.fep_lamr[s] = T.fep_has_r ? h->info[chain[w - 1]].lambda[s] : 0.0;
        }
    }
    CK(cudaMemcpy((void *)h->S.traj, h->info.data(), h->info.size() * sizeof(TrajInfo), cudaMemcpyHostToDevice));
    CK(cudaMemset(h->S.fep_acc, 0, (size_t)h->ntraj * QG_NFEP * sizeof(double)));
    for (int t = 0; t < h->ntraj; ++t) CK(cudaMemset(&h->S.tstate[t].fep_n, 0, sizeof(int)));
    h->fep_chain.assign(chain, chain + nwin);
    h->fep_kT = kT; h->fep_nskip = nskip;
    (void)L;
    return 0;
}

int qgpu_fep_result(qgpu_handle *h, double *dgf, double *dgr, double *dg, double *stats) {
    if (!h || h->fep_chain.empty()) return fail(QGPU_E_INVALID, "qgpu_fep_result: no FEP chain (qgpu_fep_start)");
    CK(cudaStreamSynchronize(h->stream));
    const int nw = (int)h->fep_chain.size();
    std::vector<double> A((size_t)h->ntraj * QG_NFEP);
    CK(cudaMemcpy(A.data(), h->S.fep_acc, A.size() * sizeof(double), cudaMemcpyDeviceToHost));
    const double rt = h->fep_kT;
    std::vector<double> f(nw, 0.0), r(nw, 0.0), g(nw, 0.0);
    for (int w = 0; w < nw; ++w) {
        const double *a = A.data() + (size_t)h->fep_chain[w] * QG_NFEP;
        const double n = a[0];
        if (w + 1 < nw) f[w] = n > 0 ? -rt * log(a[1] / n) : 0.0;
        if (w > 0) r[w] = n > 0 ? -rt * log(a[5] / n) : 0.0;
        if (stats) {
            double *o = stats + (size_t)w * 7;
            o[0] = n;
            for (int d = 0; d < 2; ++d) {
                const double s1 = a[2 + 4 * d], s2 = a[3 + 4 * d], s3 = a[4 + 4 * d];
                const double mu = n > 0 ? s1 / n : 0.0, var = n > 0 ? s2 / n - mu * mu : 0.0;
                const double m3 = n > 0 ? s3 / n - 3.0 * mu * s2 / n + 2.0 * mu * mu * mu : 0.0;
                o[1 + 3 * d] = mu;
                o[2 + 3 * d] = var;
                o[3 + 3 * d] = var > 0 ? m3 / pow(var, 1.5) : 0.0;
            }
        }
    }
    // dG(1) = 0, dG(i) = dG(i-1) + (dgf(i-1) - dgr(i))/2 (src/qfep.f90:658-661)
    for (int w = 1; w < nw; ++w) g[w] = g[w - 1] + 0.5 * (f[w - 1] - r[w]);
    if (dgf) memcpy(dgf, f.data(), nw * sizeof(double));
    if (dgr) memcpy(dgr, r.data(), nw * sizeof(double));
    if (dg) memcpy(dg, g.data(), nw * sizeof(double));
    return 0;
}

struct RowSink {
    qgpu_energies *E;
    qgpu_qenergy *EQ;
    int32_t *traj, *step;
    int32_t cap, n;
};
static void row_sink(void *user, int32_t traj, int32_t step, const qgpu_qenergy *eq, int32_t ns, const qgpu_energies *e) {
    RowSink *r = (RowSink *)user;
    if (r->n < r->cap) {
        if (r->E) r->E[r->n] = *e;
        if (r->EQ)
            for (int s = 0; s < QGPU_MAX_STATES; ++s) {
                qgpu_qenergy q{};
                if (s < ns) q = eq[s];
                r->EQ[(size_t)r->n * QGPU_MAX_STATES + s] = q;
            }
        if (r->traj) r->traj[r->n] = traj;
        if (r->step) r->step[r->n] = step;
    }
    r->n++;
}

int qgpu_run_rows(qgpu_handle *h, int32_t nsteps, int32_t ene_every, qgpu_energies *E_rows, qgpu_qenergy *EQ_rows,
                  int32_t *traj_rows, int32_t *step_rows, int32_t cap, int32_t *nrows) {
    if (!h || cap < 0 || !nrows) return fail(QGPU_E_INVALID, "qgpu_run_rows: bad arguments");
    RowSink r{E_rows, EQ_rows, traj_rows, step_rows, cap, 0};
    const int rc = qgpu_run(h, nsteps, ene_every, ene_every > 0 ? row_sink : nullptr, &r);
    *nrows = r.n;
    return rc;
}

int qgpu_run(qgpu_handle *h, int32_t nsteps, int32_t ene_every, qgpu_ene_sink sink, void *user) {
    if (!h || nsteps < 0) return fail(QGPU_E_INVALID, "bad arguments");
    if (ene_every <= 0) ene_every = 1 << 30;
    LaunchCtx L{h->stream, &h->nlaunch};
    const int NB = h->NBcycle;
    // record buffer: rows of ntraj records
    int want_cap = 256;
    if (!h->rec_d || h->rec_cap < want_cap) {
        if (h->rec_d) cudaFree(h->rec_d);
        CK(cudaMalloc(&h->rec_d, (size_t)want_cap * h->ntraj * QG_REC * sizeof(double)));
        h->rec_cap = want_cap;
        if (h->graph) { cudaGraphExecDestroy(h->graph); h->graph = nullptr; }
    }
    int ctl[2] = {(int)h->step, (int)((h->step + ene_every - 1) / ene_every)};
    launch_set_ctl(L, h->recctl_d, 2, ctl[0], ctl[1]);
    int row0 = ctl[1];
    CK(cudaMemsetAsync(h->S.fx, 0, 3 * (size_t)h->S.natom * sizeof(unsigned long long), h->stream));
    CK(cudaMemsetAsync(h->S.eacc, 0, (size_t)h->ntraj * QG_NE * sizeof(unsigned long long), h->stream));
    ensure_double(h, L);
    if (!h->temp_init) {
        // temperature() before the first step (md_run, src/md.f90:6395-6398)
        temperature_init(h, L);
        launch_finalize(h->S, L, FIN_TEMP | (h->nh_ready ? 0 : FIN_NH) | (h->all_fused ? 0 : FIN_EK64), nullptr,
                        h->zero_d, 0, 1, 0);
        h->nh_ready = 1;
        h->temp_init = 1;
    }
    bool any_file = false;
    for (FILE *f : h->ene_files) any_file = any_file || f;
    auto flush = [&](long long upto_step) -> int {
        long long rows = (upto_step + ene_every - 1) / ene_every - row0;
        if (rows > h->rec_cap) rows = h->rec_cap;
        if (rows > 0 && (sink || any_file)) {
            std::vector<double> buf((size_t)rows * h->ntraj * QG_REC);
            CK(cudaMemcpyAsync(buf.data(), h->rec_d, buf.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
            CK(cudaStreamSynchronize(h->stream));
            for (long long r = 0; r < rows; ++r)
                for (int t = 0; t < h->ntraj; ++t) {
                    const double *R = buf.data() + ((size_t)r * h->ntraj + t) * QG_REC;
                    const long long step = (row0 + r) * (long long)ene_every;
                    qgpu_energies E;
                    qgpu_qenergy EQ[QG_MAXS];
                    unpack_row(R, h->nstates[t], &E, EQ);
                    if (sink) sink(user, t, (int32_t)step, EQ, h->nstates[t], &E);
                    // qdyn writes energy frames at nonzero steps (md_run :6630)
                    if (h->ene_files[t] && step > 0) {
                        const int nod = (int)h->offd_states[t].size() / 2;
                        std::vector<int32_t> ij(2 * nod);
                        for (int q = 0; q < 2 * nod; ++q) ij[q] = h->offd_states[t][q] + 1;
                        if (qgpu_ene_write_frame(h->ene_files[t], h->nstates[t], EQ, nod, ij.data(), R + QG_REC_OD))
                            return fail(QGPU_E_INVALID, "writing the energy file of trajectory %d failed", t);
                    }
                }
        }
        return 0;
    };
    const long long end = h->step + nsteps;
    while (h->step < end) {
        const long long rows_needed = (h->step + NB + ene_every - 1) / ene_every - row0;
        if (rows_needed > h->rec_cap) {
            if (int rc = check_status(h)) return rc;
            flush(h->step);
            row0 = (int)((h->step + ene_every - 1) / ene_every);
            launch_set_ctl(L, h->recctl_d, 2, (int)h->step, row0);
        }
        if (h->step % NB == 0 && end - h->step >= NB && h->lists_built) {
            if (int rc = replay_block(h, L, ene_every)) return rc;
        } else {
            if (h->step % NB == 0) { list_ops(h, L); h->lists_built = 1; }
            step_ops(h, L, 0, ene_every, step_emode(h->step, ene_every));
            launch_tick(L, h->recctl_d, 1);
            h->step += 1;
        }
    }
    after_steps(h);
    if (int rc = check_status(h)) return rc;
    flush(h->step);
    return check_status(h);
}

}  // extern "C"
