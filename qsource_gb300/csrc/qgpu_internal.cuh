// qgpu_internal.cuh -- device-side data layout and helpers of the GB300 engine.
//
// Layout in HBM: every trajectory of a batch is concatenated.  Atoms, charge
// groups and Q atoms carry global indices; TrajInfo holds each trajectory's
// offsets and parameters.  Per-item work lists (water groups, solute atoms, ...)
// are padded per trajectory to a multiple of QG_BLOCK with -1 so that a thread
// block never spans two trajectories.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include "qgpu.h"

#define QG_BLOCK 128            // threads per block of the per-item kernels
#define QG_UBLK 96              // threads per block of the fused update (32 waters)
#define QG_LW 8                 // lanes that share one target in the pair kernels
#define QG_NSIDE 3              // side streams of the concurrent force kernels
#define QG_MAXBRANCH 8          // independent trajectory groups of a replayed block (at most)
#define QG_DEFBRANCH 4          // the groups a new handle forms
#define QG_TREG 4               // target-group atoms held in registers by the any-atom scan test
#define QG_MAXSHELL 8           // water polarisation shells per trajectory
#define QG_MAXNH 16             // Nose-Hoover chain length
#define QG_LCG_M 100000000ull   // randm modulus, multiplier (src/md.f90:17549-17551)
#define QG_LCG_MULT 31415821ull
// k_finalize flags
#define FIN_TEMP 1              // temperature() and the Berendsen scales
#define FIN_STEP 2              // a step has been taken: advance the Langevin random stream
#define FIN_NH 4                // propagate the Nose-Hoover chain for the next step
#define FIN_EK64 8              // FP64 step forms: Ekin from the int64 partials, temperatures and scales in FP64
#define QG_WPBLK 512            // threads of the water polarisation kernel (one block per trajectory)
#define S_GROUP_MASK 0xffffffffu
#define QG_MAXS 4               // states handled by the engine (<= QGPU_MAX_STATES)
#define QG_MAXQ 128             // Q atoms per trajectory (reference max_qat = 100)
#define QG_TILE_G 64            // source groups per scan tile
#define QG_TILE_A 256           // source atoms per scan tile
#ifndef QG_TPC
#define QG_TPC 1                // scan tiles per source chunk (one k_scan block)
#endif
#ifndef QG_SCAN_MINB
#define QG_SCAN_MINB 6          // k_scan register bound (minimum resident blocks)
#endif
#define QG_CAPC (QG_TPC * QG_TILE_G)  // near groups a chunk can hold (= groups in a chunk)
#define QG_MAXOD 6              // off-diagonal couplings recorded per trajectory
#define QG_NLRF 24              // LRF accumulators per group (see k_scan)
#define QG_NPHI 20              // symmetric LRF Taylor coefficients per group
#define QG_FSCALE 4294967296.0  // fixed-point scale 2^32 for forces and energies
#define QG_FMAX 1073741824.0    // |value| limit before the int64 accumulator (2^30)

// energy accumulator slots (fixed point) per trajectory
enum {
    EA_PP_EL = 0, EA_PP_VDW, EA_PW_EL, EA_PW_VDW, EA_WW_EL, EA_WW_VDW, EA_LRF,
    EA_P_BOND, EA_W_BOND, EA_P_ANG, EA_W_ANG, EA_P_TOR, EA_W_TOR, EA_P_IMP, EA_W_IMP,
    EA_RST_FIX, EA_RST_SHELL, EA_RST_RAD, EA_RST_PROT, EA_RST_WPOL,
    EA_Q0  // then per state: QB QA QT QI QQ_EL QQ_VDW QP_EL QP_VDW QW_EL QW_VDW
};
enum { EQ_B = 0, EQ_A, EQ_T, EQ_I, EQ_QQ_EL, EQ_QQ_VDW, EQ_QP_EL, EQ_QP_VDW, EQ_QW_EL, EQ_QW_VDW, EQ_RST, EQ_N };
#define QG_NE (EA_Q0 + EQ_N * QG_MAXS)
// energy record row: 29 ENERGIES + QG_MAXS*15 Q_ENERGIES + Temp, Tfree + QG_MAXOD*(Hij, rkl)
#define QG_REC_E 0
#define QG_REC_EQ 29
#define QG_REC_T (29 + 15 * QG_MAXS)
#define QG_REC_OD (QG_REC_T + 2)
#define QG_REC (QG_REC_OD + 2 * QG_MAXOD)

// status bits
#define ST_LIST_OVERFLOW 1
#define ST_SHAKE 2
#define ST_FIXED 4
#define ST_NAN 8

struct TrajInfo {
    int atom0, natom, nat_solute, nwat;
    int grp0, ncgp, ncgp_solute;
    int q0, nqat, nstates;
    int type0, natyps, lj0;     // type table offset, ljcod matrix offset
    int qlib0, nqlib, sc0;      // Q type table offset, sc_lookup offset
    int qvdw;
    int use_lrf, q_static;      // LRF on; qp/qw lists built once (Rcq > rexcl_o)
    int any_atom;               // any-atom cut-off for solute groups (iuse_switch_atom = 0)
    int tile0, ntile;           // scan tiles of this trajectory
    int nchunk;                 // source chunks of QG_TPC tiles
    long long scr0;             // first scan-scratch slot (slot = scr0 + chunk*ncgp + local group)
    int ww_lj;                  // ljcod of the water O pair
    float ww_A, ww_B;           // O-O LJ products (aLJ_solv(1,c)^2, bLJ_solv(1,c)^2)
    double ww_Ad, ww_Bd;
    // arithmetic rule with LJ on the water hydrogens (nonbon2_ww :12847,
    // nonbon2_qw :12562 take LJ on every water atom): hlj set, the products of
    // the water atom pairs [3*a+b] other than O-O (that one is ww_A/ww_B, and
    // entry 0 is zero), and the sc_lookup columns of the two H (their types)
    int hlj;
    float wwh_A[9], wwh_B[9];
    double wwh_Ad[9], wwh_Bd[9];
    int wh_col[2];
    float chg_solv[3];
    float wwqq[9];              // chg_solv(a)*chg_solv(b), nonbond_ww_spc charge products
    float el14;
    double el14d;
    float rc2_pp, rc2_pw, rc2_ww, rc2_lrf;   // float prefilter thresholds
    double drc2_pp, drc2_pw, drc2_ww, drc2_lrf, drcq2;
    double origin[3];           // float coordinates are relative to this point
    double xpcent[3], xwcent[3];
    double rwat, fk_wsphere, Dwmz, awmz, fk_pshell, fk_fix;
    double lambda[QG_MAXS];
    float lambdaf[QG_MAXS];
    double dt, Temp0, tau_T, inv_dt;
    float dtf, inv_dtf;
    // temperature(): T = Ekin * c, c = 2/(Boltz*Ndegf...); dt/tau_T; Temp0
    float cT, cTfree, cTfsu, cTfsv, dt_tau, Temp0f;
    double dt_taud;             // dt/tau_T in FP64 (the FP64 step forms)
    // float copies of the restraint parameters for the per-step kernels
    float fk_wspheref, rwatf, Dwmzf, awmzf, fk_pshellf, fk_fixf;
    int separate_scaling, detail_temps;
    int Ndegf, Ndegfree, Ndegfree_solute, Ndegfree_solvent;
    int shake_mol0, nshake_mol;
    int nb0[6], nbn[6];         // bonded term ranges: p/w bonds, p/w angles... (see host)
    int qq0[QG_MAXS], nqq[QG_MAXS];
    int qterm0[4], nqterm[4];   // Q bond/angle/torsion/improper ranges
    int ekin_blk0, ekin_nblk;   // Ekin partial slots of this trajectory (update blocks)
    int ff_type;
    // water polarisation restraint (watpol): shells, layer bound, first of
    // this trajectory's wpol state slots (-1 when off)
    int wpol, nshell, wp0, freeze;
    double fkwpol, wp_rlayer;
    double sh_rout[QG_MAXSHELL], sh_cstb[QG_MAXSHELL], sh_acos_cstb[QG_MAXSHELL];
    int itdis_update;
    // thermostat (0 Berendsen, 1 Langevin, 2 Nose-Hoover) and integrator
    // (0 leap-frog, 1 velocity-verlet); dv_mod = dt or dt/2 (md_run :6440-6460)
    int thermostat, integrator, lgauss, nhc;
    double dvm, lfric, kbT;
    double dvm_q;                    // dvm * 2^-32: the fixed-point gradient's unit folded in (exact)
    float dvmf, lfricf;
    unsigned long long lcgA, lcgC;   // randm stream advance of one step (3N or 36N numbers)
    double qnh[QG_MAXNH];
    // free-energy perturbation (qfep Part 1) on the device: this trajectory's
    // window has neighbours (has_f / has_r) with lambdas lamf / lamr
    int fep_on, fep_has_f, fep_has_r, fep_nskip;
    double fep_kT, fep_lamf[QG_MAXS], fep_lamr[QG_MAXS];
    // periodic box (use_pbc): edges and inverse edges, the Q switching atom
    // (global index), the molecules put_back_in_box may move (DevSys::mol_start
    // from mol0, nmol of them, the first nsolute_mol solute) and which kinds
    int pbc, qswitch, put_solute, put_solvent, rigid_box;
    // combination rule: 0 geometric (A = a_i a_j), 1 arithmetic (ivdw_rule 2,
    // nonbon2_*: A = b_i b_j (a_i + a_j)^12, B = 2 b_i b_j (a_i + a_j)^6)
    int arith;
    int mol0, nmol, nsolute_mol;
    float boxf[3], iboxf[3];
    double box[3], ibox[3];
};
#define QG_NFEP 9                // FEP accumulators per trajectory (see k_finalize)

// Records the message for qgpu_last_error and returns code (qgpu_api.cu).
int qgpu_fail(int code, const char *fmt, ...);
// Q energy-file records (qgpu_ene.cu): header, and one frame (nstates
// state records + the OFFD record; offd_ij 1-based state pairs, offd_Hr
// (Hij, rkl) per coupling)
int qgpu_ene_write_header(FILE *f, const char *version);
int qgpu_ene_write_frame(FILE *f, int32_t nstates, const qgpu_qenergy *EQ, int32_t noffd, const int32_t *offd_ij,
                         const double *offd_Hr);

// Per-trajectory dynamic state (device).
// Per-trajectory dynamic state (device), in FP32: it is updated every step by
// a one-warp kernel, where each FP64 instruction would hold the FP64 pipe for
// ~64 cycles of a serial chain.
struct TrajState {
    float Temp, Tfree, Ekin;
    float tsf_solute, tsf_solvent;  // Berendsen scales of the next step
    float wshiftf;                  // sqrt(Boltz*Tfree/fk_wsphere), restrain_solvent
    int shake_iters;                // SHAKE sweeps (molecule sweeps) since the counter was read
    int shake_visits;               // constraint visits of the FP64 fused step's SHAKE (same)
    unsigned rnd;                   // randm state before the next step's random forces
    int fep_n;                      // recorded frames seen by the FEP accumulation
    double nh_s1, nh_s2;            // Nose-Hoover velocity scales of the next step
    // FP64 copies: formed in FP64 from the int64 Ekin partials in the FP64
    // step forms (FIN_EK64), widened from the float values otherwise
    double Ekin_d, Temp_d, Tfree_d;
    double tsd_solute, tsd_solvent; // Berendsen scales of the next step
};

struct DevSys {
    int ntraj, natom, ngrp, nq;
    int nb_cap;
    const TrajInfo *traj;
    TrajState *tstate;
    // atoms
    double *x, *v, *xx;
    const double *xtop, *winv, *mass;
    float4 *pos, *poslo;            // hi part + charge, lo part
    // The fused MD path keeps its master state in float: pos/poslo as a
    // double-float (about 48 significant bits) relative to the trajectory
    // origin, and float velocities.  x/v are refreshed from it when a step
    // or an API call reads them (see k_update_f and k_sync_double).
    float4 *velf;
    const float *winvf, *massf;
    const float4 *xtoph, *xtopl;    // topology coordinates relative to the origin, hi/lo
    // packed water record at the slots of each water's 3 atoms (O first):
    //   [O] = (O_hi.xyz, d1.x)  [O+1] = (O_lo.xyz, d1.y)  [O+2] = (d1.z, d2.xyz)
    // with dk = H_k - O in float: a neighbour water is 3 float4 loads.
    float4 *wrec;
    const int *atype;               // global type index
    const double *crg_d;            // scaled charges (FP64)
    const int *aq;                  // global Q index or -1
    const uint8_t *aexcl, *ashell;
    const int *atraj, *agrp;
    unsigned long long *fx;         // 3*natom fixed-point gradient
    const unsigned long long *exmask, *p14mask;  // solute exclusion / 1-4 bits, offsets -32..31
    const int *exlong_first, *exlong_j, *exlong_kind;
    // types
    const float *avdw, *bvdw;       // [type*3 + code-1]
    const double *avdw_d, *bvdw_d;
    const int8_t *ljcod;            // per-trajectory matrices at TrajInfo::lj0
    // groups
    const int *g_start, *g_atoms, *g_switch, *g_kind, *g_traj;
    const uint8_t *g_excl;
    double *g_cent;                 // 3*G
    float4 *g_centf;                // centre - origin in float (per list build)
    float *g_phi;                   // QG_NLRF*G accumulators
    float *g_phif;                  // QG_NPHI*G Taylor coefficients
    // neighbour list of a group: water neighbours first (as their O atom),
    // then solute neighbours (as group index); nb_nw = number of water entries
    int *nb_count, *nb_nw, *nb_list;
    const int *tile_g0, *tile_g1;
    // scan scratch (per slot = (chunk, target group)): FP32 LRF partial sums,
    // near-group count and near groups of the chunk
    float *scr_phi;                 // QG_NLRF per slot
    int *scr_cnt;                   // per slot
    int *scr_nb;                    // QG_CAPC per slot
    // periodic box with any-atom lists only (else null): per neighbour entry
    // the atom pair that fixes the group pair's periodic shift (the first pair
    // inside the cut-off in the reference's loop order: nbpp_cgp / nbpw_cgp of
    // nbpplis2_box_lrf and nbpwlis2_box_lrf), (atom of the list's own group,
    // atom of the neighbour); parallel to nb_list and to scr_nb
    int2 *nb_sha = nullptr, *scr_sha = nullptr;
    // Q atoms
    const int *q_atom;              // global atom of each global Q index
    const float *qcrg_f;            // [q*QG_MAXS+s]
    const double *qcrg_d;
    const int *qiac;                // [q*QG_MAXS+s] global Q-type index
    const float *qavdw, *qbvdw;     // [qtype*3 + code-1]
    const double *qavdw_d, *qbvdw_d;
    const float *sc_f;              // sc_lookup, [(q*(natyps+nqat)+col)*QG_MAXS+s] at TrajInfo::sc0
    const double *sc_d;
    float *qw_A, *qw_B;             // [q*QG_MAXS+s] water-O LJ products
    const double *qw_Ad, *qw_Bd;
    const int *qw_lj;               // [q] LJ code of the water-O / Q-atom pair
    const int *qw_sc;               // [q] sc_lookup column of the water O (the LJ code, or its type: arithmetic rule)
    // arithmetic rule with LJ on the water hydrogens: [(q*QG_MAXS+s)*2 + h]
    // LJ products of Q atom q in state s with water H h (0, 1); null otherwise
    const float *qwh_A, *qwh_B;
    const double *qwh_Ad, *qwh_Bd;
    // LJ products per (type pair, code) under the trajectory's combination
    // rule, [(lj0 + ta*natyps + tb)*3 + code-1] (lj_index)
    const float *ljA, *ljB;
    const double *ljA_d, *ljB_d;
    uint8_t *qw_member;             // per water (global water index) in the qw list
    uint8_t *qp_member;             // per atom in the qp list
    int *g_qin;                     // per solute group in a box: the atom that put it on the qp list (its shift)
    const int *mol_start;           // molecules of the box trajectories: first atom (global); TrajInfo::mol0
    double *boxc;                   // per trajectory: box centre (put_back_in_box)
    // the other p_restrain restraints, one item each (wall restraints one per
    // atom), padded per trajectory to blocks of QG_BLOCK: kind (-1 padding, 0
    // position, 1 distance, 2 angle, 3 wall), atoms[3], state (0 = all),
    // parameters xr_p[6] (FP64) / xr_pf[9] (float; positions as hi/lo offsets)
    const int *xr_kind, *xr_at, *xr_st, *xr_blk_traj;
    const double *xr_p;
    const float *xr_pf;
    int nxr;
    const uint8_t *qp_skip;
    const int *qp14_first, *qp14_q; // per atom CSR of Q atoms with qconn == 4
    // nbqq
    const int *qq_iq, *qq_j, *qq_jq; const int8_t *qq_lj; const double *qq_els; const float *qq_elsf;
    // Q bonded terms (flattened per kind, codes already per state)
    const int *qt_atoms;            // 4 atoms per term
    const int *qt_cod;              // [term*QG_MAXS+s] 1-based lib index (global) or 0
    const int *qt_kind, *qt_traj;   // 0 bond 1 angle 2 torsion 3 improper
    const double *qt_lib;           // 4 doubles per lib entry
    const float *qt_libf;
    int nqt;
    // classical bonded terms
    const int *bt_atoms;            // 4 atoms per term
    const int *bt_cod;              // global lib index (0-based)
    const double *bt_lib;           // 4 doubles per entry
    const float *bt_libf;
    const int *bt_kind;             // 0 bond 1 angle 2 torsion 3 harmonic improper 4 periodic improper
    int nbt;                        // padded term list; blocks are single (trajectory, slot)
    const int *bt_blk_traj, *bt_blk_slot;
    // off-diagonal couplings
    const int *od_traj, *od_ij, *od_kl; const double *od_Amu; int nod;
    double *od_out;                 // [traj][QG_MAXOD][2]: Hij, rkl
    // shake
    const int *shk_first, *shk_i, *shk_j, *shk_traj;
    const double *shk_d2;
    const float2 *shk_d2hl;         // d0^2 as a float pair (hi, lo)
    int nshk_mol;
    // sequence restraints (p_restrain): atom range [rs_i0, rs_i1], force
    // constant, H flag, to_centre, trajectory
    const int *rs_i0, *rs_i1, *rs_ih, *rs_tc, *rs_traj;
    const double *rs_fk;
    int nrs;
    const uint8_t *aheavy;
    // Langevin: random-force amplitude sqrt(gkT/winv) per atom; skip-ahead of
    // the randm stream to each atom's first number: x_atom = (A x + C) mod m
    const double *randva;
    const float *randvaf;
    const unsigned *lcg_a, *lcg_c;
    double *nh_state;               // per trajectory: vnh[QG_MAXNH], xnh[QG_MAXNH]
    double *fep_acc;                // per trajectory: QG_NFEP sums (k_finalize)
    int *fin_cnt;                   // per trajectory: update blocks done this step (fused step end)
    // water polarisation state per (trajectory, shell): theta_corr, avtheta,
    // avn_insh (slot = TrajInfo::wp0 + shell)
    double *wp_state;               // 3 doubles per slot
    // energies and reductions
    unsigned long long *eacc;       // QG_NE per trajectory
    float *ekin_part;               // 4 per Ekin block
    long long *ekin_fx;             // 4 per Ekin block: fixed-point (2^-32 kcal/mol) partials, FP64 step forms
    int *status;
};

// ------------------------------------------------------------- helpers
__device__ __forceinline__ void fx_add(unsigned long long *p, double v, int *status) {
    if (!(fabs(v) < QG_FMAX)) { atomicOr(status, ST_FIXED); return; }
    long long q = __double2ll_rn(v * QG_FSCALE);
    atomicAdd(p, (unsigned long long)q);
}
__device__ __forceinline__ double fx_get(unsigned long long u) { return (double)(long long)u * (1.0 / QG_FSCALE); }

// round(v * 2^32) as an int64 from the float's bits, with integer
// instructions only: on GB300 the FP64 pipe (which also converts to and from
// double) issues at 1/64 of the FP32 rate, so per-atom epilogues avoid it.
// Ties round away from zero.  Callers keep |v| < 2^30.
__device__ __forceinline__ long long f2fx(float v) {
    const unsigned u = __float_as_uint(v);
    const int e = (int)((u >> 23) & 0xffu);
    if (e == 0) return 0;                                       // zero / subnormal
    const unsigned long long m = (u & 0x7fffffu) | 0x800000u;   // |v| = m * 2^(e-150)
    int sh = e - 118;                                           // |v| * 2^32 = m * 2^sh
    if (sh > 38) sh = 38;
    unsigned long long r;
    if (sh >= 0) r = m << sh;
    else if (sh >= -24) r = (m + (1ull << (-sh - 1))) >> (-sh);
    else r = 0;
    return (u >> 31) ? -(long long)r : (long long)r;
}
// the fixed-point gradient from a float (no FP64 instruction)
__device__ __forceinline__ void fx_addf(unsigned long long *p, float v, int *status) {
    if (!(fabsf(v) < 1073741824.f)) { atomicOr(status, ST_FIXED); return; }
    atomicAdd(p, (unsigned long long)f2fx(v));
}
// fixed-point value of a float with the range check
__device__ __forceinline__ long long f2fx_chk(float v, int *status) {
    if (!(fabsf(v) < 1073741824.f)) { atomicOr(status, ST_FIXED); return 0; }
    return f2fx(v);
}
__device__ __forceinline__ long long d2fx_chk(double v, int *status) {
    if (!(fabs(v) < QG_FMAX)) { atomicOr(status, ST_FIXED); return 0; }
    return __double2ll_rn(v * QG_FSCALE);
}
// float value of a fixed-point accumulator without FP64: the high word holds
// the integer part, the low word 2^-32 units
__device__ __forceinline__ float fx_getf(unsigned long long u) {
    const long long q = (long long)u;
    return (float)(int)(q >> 32) + (float)(unsigned)(q & 0xffffffffull) * 2.3283064365386963e-10f;
}

// compensated float accumulation (Kahan)
struct KSum {
    float s, c;
    __device__ __forceinline__ void zero() { s = 0.f; c = 0.f; }
    __device__ __forceinline__ void add(float v) {
        float y = v - c;
        float t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ __forceinline__ double value() const { return (double)s - (double)c; }
    // fixed-point value of scale * (s - c)
    __device__ __forceinline__ long long fx(float scale, int *status) const {
        return f2fx_chk(s * scale, status) - f2fx_chk(c * scale, status);
    }
};

// Block sums of N int64 fixed-point energies into the slots of one
// trajectory: warp shuffles, then warp 0 adds the warps' partials in order.
// Every thread of the block must call it.
template <int N>
__device__ __forceinline__ void block_energies_fx(unsigned long long *eacc, const int (&slot)[N], long long (&v)[N],
                                                  long long (*red)[QG_BLOCK / 32]) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < N; ++k)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < N; ++k) red[k][warp] = v[k];
    __syncthreads();
    if (threadIdx.x < N) {
        long long s = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[threadIdx.x][w];
        int sl = 0;
#pragma unroll
        for (int k = 0; k < N; ++k) sl = (k == (int)threadIdx.x) ? slot[k] : sl;   // no local-memory indexing
        if (s) atomicAdd(eacc + sl, (unsigned long long)s);
    }
}

__device__ __forceinline__ double warp_sum_d(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
// Error-free transformations (Knuth two-sum, Dekker fast two-sum; FMA two-product)
__device__ __forceinline__ float two_sum(float a, float b, float &err) {
    const float s = a + b, bb = s - a;
    err = (a - (s - bb)) + (b - bb);
    return s;
}
__device__ __forceinline__ float fast_two_sum(float a, float b, float &err) {   // |a| >= |b|
    const float s = a + b;
    err = b - (s - a);
    return s;
}
__device__ __forceinline__ float two_prod(float a, float b, float &err) {
    const float p = a * b;
    err = fmaf(a, b, -p);
    return p;
}
__device__ __forceinline__ float warp_sum_f(float v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// hi/lo float difference: (b - a) with the rounding error of the absolute
// coordinates removed
__device__ __forceinline__ float3 dpos(const float4 ah, const float4 al, const float4 bh, const float4 bl) {
    return make_float3((bh.x - ah.x) + (bl.x - al.x), (bh.y - ah.y) + (bl.y - al.y), (bh.z - ah.z) + (bl.z - al.z));
}

// Packed record of one water (see DevSys::wrec) from its hi/lo coordinates:
// float4 number k (0..2) of the record.
__device__ __forceinline__ float4 wrec_part(const float4 (&h)[3], const float4 (&l)[3], int k) {
    float d[2][3];
#pragma unroll
    for (int m = 1; m < 3; ++m) {
        d[m - 1][0] = (h[m].x - h[0].x) + (l[m].x - l[0].x);
        d[m - 1][1] = (h[m].y - h[0].y) + (l[m].y - l[0].y);
        d[m - 1][2] = (h[m].z - h[0].z) + (l[m].z - l[0].z);
    }
    if (k == 0) return make_float4(h[0].x, h[0].y, h[0].z, d[0][0]);
    if (k == 1) return make_float4(l[0].x, l[0].y, l[0].z, d[0][1]);
    return make_float4(d[0][2], d[1][0], d[1][1], d[1][2]);
}
__device__ __forceinline__ void put_wrec(float4 *wr, const float4 (&h)[3], const float4 (&l)[3]) {
#pragma unroll
    for (int k = 0; k < 3; ++k) wr[k] = wrec_part(h, l, k);
}
// randm (src/md.f90:17543-17577): irand <- (irand*31415821 + 1) mod 10^8,
// r = 10*(irand/10)/10^8
__device__ __forceinline__ unsigned lcg_next(unsigned x) {
    return (unsigned)(((unsigned long long)x * QG_LCG_MULT + 1ull) % QG_LCG_M);
}
__device__ __forceinline__ double lcg_real(unsigned x) {
    const double r = (double)(x / 10u) * 10.0 / 100000000.0;
    return (r <= 0.0 || r > 1.0) ? 0.0 : r;
}
// Langevin random force of atom a for this step (newvel_lan, src/md.f90:
// 6232-6247): uniform randva*(r - 1/2) or Gaussian gauss(0, randva), from the
// atom's own position in the step's stream.
template <typename R>
__device__ __forceinline__ void langevin_force(const DevSys &S, const TrajInfo &T, unsigned base, int a, R (&f)[3]) {
    unsigned x = (unsigned)(((unsigned long long)S.lcg_a[a] * base + S.lcg_c[a]) % QG_LCG_M);
    const R amp = sizeof(R) == 8 ? R(S.randva[a]) : R(S.randvaf[a]);
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        if (!T.lgauss) {
            x = lcg_next(x);
            f[j] = amp * (R(lcg_real(x)) - R(0.5));
        } else {
            double s = 0.0;
            for (int q = 0; q < 12; ++q) { x = lcg_next(x); s += lcg_real(x); }
            f[j] = R(s - 6.0) * amp;
        }
    }
}
// Periodic box.  The shift of a difference d is L*nint(d/L) per component
// (boxlength*nint(d*inv_boxl), every box routine of src/md.f90); the float
// form rounds to nearest-even, which differs from nint only at exact
// half-integers (components of exactly half a box, far outside every cut-off).
__device__ __forceinline__ float3 box_shift(const TrajInfo &T, const float3 d) {
    return make_float3(T.boxf[0] * rintf(d.x * T.iboxf[0]), T.boxf[1] * rintf(d.y * T.iboxf[1]),
                       T.boxf[2] * rintf(d.z * T.iboxf[2]));
}
__device__ __forceinline__ float3 f3sub(const float3 a, const float3 b) {
    return make_float3(a.x - b.x, a.y - b.y, a.z - b.z);
}
// FP64 shift of x[b] - x[a] in the reference's operation order
__device__ __forceinline__ double3 box_shift_d(const TrajInfo &T, const double *x, int a, int b) {
    double3 s;
    s.x = __dmul_rn(T.box[0], round(__dmul_rn(__dsub_rn(x[3 * b], x[3 * a]), T.ibox[0])));
    s.y = __dmul_rn(T.box[1], round(__dmul_rn(__dsub_rn(x[3 * b + 1], x[3 * a + 1]), T.ibox[1])));
    s.z = __dmul_rn(T.box[2], round(__dmul_rn(__dsub_rn(x[3 * b + 2], x[3 * a + 2]), T.ibox[2])));
    return s;
}
// exact FP64 minimum-image squared distance (nbpplist_box_lrf src/md.f90:
// 8282-8288: dx = dx - boxlength*nint(dx*inv_boxl), r2 = dx**2+dy**2+dz**2)
__device__ __forceinline__ double dist2_exact_box(const double *x, int i, int j, const TrajInfo &T) {
    double c[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const double a = __dsub_rn(x[3 * i + k], x[3 * j + k]);
        c[k] = __dsub_rn(a, __dmul_rn(T.box[k], round(__dmul_rn(a, T.ibox[k]))));
    }
    return __dadd_rn(__dadd_rn(__dmul_rn(c[0], c[0]), __dmul_rn(c[1], c[1])), __dmul_rn(c[2], c[2]));
}

// index of the LJ products of local types (ta, tb), code c (1..3), in DevSys::ljA/ljB
__device__ __forceinline__ int lj_index(const TrajInfo &T, int ta, int tb, int c) {
    return (T.lj0 + (ta - T.type0) * T.natyps + (tb - T.type0)) * 3 + c - 1;
}

// exact FP64 squared distance in the reference's operation order (no FMA)
__device__ __forceinline__ double dist2_exact(const double *x, int i, int j) {
    double a = __dsub_rn(x[3 * i], x[3 * j]);
    double b = __dsub_rn(x[3 * i + 1], x[3 * j + 1]);
    double c = __dsub_rn(x[3 * i + 2], x[3 * j + 2]);
    return __dadd_rn(__dadd_rn(__dmul_rn(a, a), __dmul_rn(b, b)), __dmul_rn(c, c));
}

// ---------------------------------------------------------- launchers
struct KernelProfiler;
struct LaunchCtx {
    cudaStream_t stream;
    long long *nlaunch;
    KernelProfiler *prof = nullptr;   // per-kernel CUDA-event timing when set
};
// bracket one launch with CUDA events on L.stream (no-ops without a profiler)
void prof_begin(LaunchCtx &L, const char *name);
void prof_end(LaunchCtx &L);
// Launch-shape choices of the pair kernels (the autotuner's parameters);
// 0 = default.
struct Tuning {
    int lw_water = 8, minb_water = 1, lw_solute = 8, lg_qw = 0, unroll_water = 2;
};
struct BlockTables {
    Tuning tune;
    // per-item lists (padded per trajectory to QG_BLOCK)
    const int *wgrp; int nwgrp;        // water groups
    const int *satom; int nsatom;      // solute atoms (all, incl. Q/excluded -> skipped in kernels)
    const int *scan_t0; const int *scan_tn; const int *scan_traj; const int *scan_chunk; int nscan;  // scan blocks
    const int *gall; int ngall;        // all groups (centres)
    const int *uitem; int nuitem;      // update items (atoms, or (1<<30)|shake molecule), padded
    // fused update, one thread per atom in blocks of QG_UBLK: unconstrained
    // atoms first, then 32 waters (96 atoms) per block; ucon = first
    // constraint of the water whose first atom is in that slot, else -1
    const int *uatom, *ucon; const uint8_t *ublk_water; int nuatom;
    const int *qqblk_traj, *qqblk_s; int nqqblk;
    int max_nqat;                      // largest Q-atom count of a trajectory
    // water polarisation: trajectories with the restraint, their scratch
    const int *wp_traj, *wp_scr0; double *wp_scr; int nwp;
    int any_atom;                      // some trajectory uses the any-atom cut-off
    int pbc;                           // some trajectory is a periodic box
    int hlj;                           // some trajectory has LJ on the water hydrogens (arithmetic rule)
    // put_back_in_box: one block per trajectory that moves molecules
    const int *pb_traj; int npb;
    int nxrblk;                        // blocks of the p_restrain items (DevSys::xr_*)
    // The trajectories a set of tables covers: the whole batch, or one group
    // of consecutive trajectories whose kernels run as an independent branch
    // of the replayed graph (the list pointers above then point into the
    // group's part of each list).  Charge groups [g0, g0 + ng); the first
    // fused-update block (Ekin slot base); Q bonded terms [qt0, qt0 + nqt);
    // off-diagonal items [od0, od0 + nod); classical bonded blocks from bt0;
    // sequence restraints from rs0; p_restrain item blocks from xr0.
    int g0 = 0, ng = 0, ublk0 = 0, qt0 = 0, nqt = 0, od0 = 0, nod = 0, bt0 = 0, nbtblk = 0, rs0 = 0, nrs = 0,
        xr0 = 0;
};

void launch_centers(const DevSys &S, const BlockTables &B, LaunchCtx &L);
void launch_scan(const DevSys &S, const BlockTables &B, LaunchCtx &L);
void launch_qmember(const DevSys &S, const BlockTables &B, LaunchCtx &L, int first);
// put_back_in_box (src/md.f90:18740-18857) of the box trajectories, before a list build of the MD loop
void launch_put_back(const DevSys &S, const BlockTables &B, LaunchCtx &L);
// Energy accuracy: EACC_FP32 sums FP32 pair energies (Kahan + FP64 block
// sums); EACC_FP64 evaluates every pair energy in FP64 from the master
// coordinates (forces are FP32 in both); EACC_RECORD uses FP64 on the steps
// whose energies are recorded (step = recctl[0] + k, step % ene_every == 0).
enum { EACC_FP32 = 0, EACC_FP64 = 1, EACC_RECORD = 2 };
struct EaccSel {
    int mode;
    const int *recctl;
    int k, ene_every;
};
// pair-energy mode of the water and solute pair kernels: FP32 Kahan sums,
// FP64 terms (drop-in calls), or none (MD steps whose energies are not recorded)
enum { QG_PAIR_E_FP32 = 0, QG_PAIR_E_FP64 = 1, QG_PAIR_E_NONE = 2 };
void launch_nb_water(const DevSys &S, const BlockTables &B, LaunchCtx &L, int lrf, int emode);
void launch_nb_solute(const DevSys &S, const BlockTables &B, LaunchCtx &L, int lrf, int emode);
void launch_qw(const DevSys &S, const BlockTables &B, LaunchCtx &L, EaccSel e, int emode);
void launch_qp(const DevSys &S, const BlockTables &B, LaunchCtx &L, EaccSel e, int emode);
// nonbond_qq, Q bonded, classical bonded, restraints and off-diagonals in one launch
// On each launch the kernel evaluates in FP64 from x when eacc_on(e), else in
// FP32 from the float coordinates.
void launch_misc(const DevSys &S, const BlockTables &B, LaunchCtx &L, int terms, EaccSel e);
void launch_watpol(const DevSys &S, const BlockTables &B, LaunchCtx &L, EaccSel e);
void launch_integrate(const DevSys &S, const BlockTables &B, LaunchCtx &L);
void launch_shake(const DevSys &S, const BlockTables &B, LaunchCtx &L, int traj_filter);
void launch_update(const DevSys &S, const BlockTables &B, LaunchCtx &L, int mode);
// the fused step with the float master; writes x/v as well when the next
// step lists or records (e: the record selector of this step, nbcycle)
void launch_update_f(const DevSys &S, const BlockTables &B, LaunchCtx &L, EaccSel e, int nbcycle, int ekin_only,
                     int fin = 0, double *rec = nullptr, int rec_cap = 0);
// the fused step with the FP64 master (x, v, leap-frog and SHAKE in FP64)
void launch_update_d(const DevSys &S, const BlockTables &B, LaunchCtx &L, EaccSel e, int ekin_only, int fin = 0,
                     double *rec = nullptr, int rec_cap = 0);
// x = origin + hi + lo, v = velf for every atom
void launch_sync_double(const DevSys &S, const BlockTables &B, LaunchCtx &L);
void launch_finalize(const DevSys &S, LaunchCtx &L, int do_temperature, double *rec, const int *rec_base, int k,
                     int ene_every, int rec_cap);
void launch_tick(LaunchCtx &L, int *rec_base, int n);
void launch_set_ctl(LaunchCtx &L, int *ctl, int n, int a, int b = 0);   // ctl[0] = a, and ctl[1] = b when n > 1
void launch_mirror(const DevSys &S, const BlockTables &B, LaunchCtx &L);   // also refreshes wrec
void launch_wrec(const DevSys &S, const BlockTables &B, LaunchCtx &L);
void launch_mirror_range(const DevSys &S, LaunchCtx &L, int a0, int n);   // one trajectory's atoms
void launch_grad_to_double(const DevSys &S, LaunchCtx &L, double *out, int atom0, int natom);
