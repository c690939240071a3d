// k_small.cu -- the small FP64 terms of pot_energy (src/md.f90:16100-16150):
// nonbond_qq, the per-state Q bonded terms, classical bonded terms, the sphere
// restraints and the EVB off-diagonal couplings.  These are O(Q^2) or O(N)
// with little arithmetic, so they stay in FP64 like the reference.
#include <math.h>

#include "qgpu_internal.cuh"

#define QREAL_EPS 1.0e-14   // src/sizes.f90:48
#define BOLTZ 0.001986      // src/md.f90:54

__device__ __forceinline__ void block_energy_d(const DevSys &S, int traj, int slot, double v, double *red) {
    v = warp_sum_d(v);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += red[k];
        if (s != 0.0) fx_add(S.eacc + (size_t)traj * QG_NE + slot, s, S.status);
    }
}
__device__ __forceinline__ void grad_add(const DevSys &S, int a, double gx, double gy, double gz) {
    fx_add(S.fx + 3 * a, gx, S.status);
    fx_add(S.fx + 3 * a + 1, gy, S.status);
    fx_add(S.fx + 3 * a + 2, gz, S.status);
}

// nonbond_qq, src/md.f90:13491-13636.  One block per (trajectory, state).
__device__ void qq_block(const DevSys &S, int b, const int *blk_traj, const int *blk_s, double *red) {
    const int traj = blk_traj[b], s = blk_s[b];
    const TrajInfo &T = S.traj[traj];
    const double lam = T.lambda[s];
    const int ntq = T.natyps + T.nqat;
    double eqq_el = 0, eqq_vdw = 0, eqp_el = 0, eqp_vdw = 0;
    for (int k = T.qq0[s] + threadIdx.x; k < T.qq0[s] + T.nqq[s]; k += blockDim.x) {
        const int q = S.qq_iq[k], i = S.q_atom[q], j = S.qq_j[k], jq = S.qq_jq[k], c = S.qq_lj[k];
        const int iql = q - T.q0;
        const double qi = S.qcrg_d[q * QG_MAXS + s];
        double qj, aLJ, bLJ;
        if (!T.qvdw) {
            const int ti = S.atype[i], tj = S.atype[j];
            aLJ = S.avdw_d[ti * 3 + c - 1] * S.avdw_d[tj * 3 + c - 1];
            bLJ = S.bvdw_d[ti * 3 + c - 1] * S.bvdw_d[tj * 3 + c - 1];
            qj = jq >= 0 ? S.qcrg_d[jq * QG_MAXS + s] : S.crg_d[j];
        } else {
            const int ti = S.qiac[q * QG_MAXS + s];
            aLJ = S.qavdw_d[ti * 3 + c - 1];
            bLJ = S.qbvdw_d[ti * 3 + c - 1];
            if (jq >= 0) {
                const int tj = S.qiac[jq * QG_MAXS + s];
                aLJ *= S.qavdw_d[tj * 3 + c - 1];
                bLJ *= S.qbvdw_d[tj * 3 + c - 1];
                qj = S.qcrg_d[jq * QG_MAXS + s];
            } else {
                if (c == 2) { aLJ = S.qavdw_d[ti * 3]; bLJ = S.qbvdw_d[ti * 3]; }
                const int tj = S.atype[j];
                aLJ *= S.avdw_d[tj * 3 + c - 1];
                bLJ *= S.bvdw_d[tj * 3 + c - 1];
                qj = S.crg_d[j];
            }
        }
        const double dx = S.x[3 * j] - S.x[3 * i], dy = S.x[3 * j + 1] - S.x[3 * i + 1], dz = S.x[3 * j + 2] - S.x[3 * i + 2];
        double r2 = dx * dx + dy * dy + dz * dz;
        const double r6hc = r2 * r2 * r2;
        // softcore column natyps+jq, natyps for a non-Q partner (src/md.f90:13561)
        const int col = jq >= 0 ? T.natyps + (jq - T.q0) : T.natyps - 1;
        double r6 = r6hc + S.sc_d[(size_t)T.sc0 + ((size_t)iql * ntq + col) * QG_MAXS + s];
        r6 = 1.0 / r6;
        const double r12 = r6 * r6;
        r2 = 1.0 / r2;
        const double r = sqrt(r2);
        double Vel = qi * qj * r * S.qq_els[k];
        if (c == 3) Vel *= T.el14;
        double Va, Vb, dv;
        if (T.qvdw && jq >= 0 && c == 2) {
            Va = aLJ * exp(-bLJ / r);
            Vb = 0.0;
            dv = r2 * (-Vel - bLJ * Va / r) * lam;
        } else {
            Va = aLJ * r12;
            Vb = bLJ * r6;
            dv = r2 * (-Vel - (12.0 * Va - 6.0 * Vb) * r6hc * r6) * lam;
        }
        grad_add(S, i, -dv * dx, -dv * dy, -dv * dz);
        grad_add(S, j, dv * dx, dv * dy, dv * dz);
        if (jq >= 0) { eqq_el += Vel; eqq_vdw += Va - Vb; }
        else { eqp_el += Vel; eqp_vdw += Va - Vb; }
    }
    const int base = EA_Q0 + EQ_N * s;
    block_energy_d(S, traj, base + EQ_QQ_EL, eqq_el, red);
    block_energy_d(S, traj, base + EQ_QQ_VDW, eqq_vdw, red);
    block_energy_d(S, traj, base + EQ_QP_EL, eqp_el, red);
    block_energy_d(S, traj, base + EQ_QP_VDW, eqp_vdw, red);
}

// --------------------------------------------------- angle / dihedral
__device__ double angle_grad(const DevSys &S, int i, int j, int k, double fk, double ang0, double scale, double gi[3],
                             double gk[3]) {
    double rji[3], rjk[3];
    for (int a = 0; a < 3; ++a) { rji[a] = S.x[3 * i + a] - S.x[3 * j + a]; rjk[a] = S.x[3 * k + a] - S.x[3 * j + a]; }
    const double bji = sqrt(rji[0] * rji[0] + rji[1] * rji[1] + rji[2] * rji[2]);
    const double bjk = sqrt(rjk[0] * rjk[0] + rjk[1] * rjk[1] + rjk[2] * rjk[2]);
    double scp = (rji[0] * rjk[0] + rji[1] * rjk[1] + rji[2] * rjk[2]) / (bji * bjk);
    scp = fmin(1.0, fmax(-1.0, scp));
    const double ang = acos(scp), da = ang - ang0;
    const double dv = fk * da * scale;
    double f1 = sin(ang);
    if (fabs(f1) < QREAL_EPS) f1 = QREAL_EPS;
    f1 = -1.0 / f1;
    for (int a = 0; a < 3; ++a) {
        gi[a] = dv * f1 * (rjk[a] / (bji * bjk) - scp * rji[a] / (bji * bji));
        gk[a] = dv * f1 * (rji[a] / (bji * bjk) - scp * rjk[a] / (bjk * bjk));
    }
    return 0.5 * fk * da * da;
}

// dihedral angle and its derivative components (src/md.f90:17241-17538)
__device__ double dihedral(const DevSys &S, int i, int j, int k, int l, double dp[12]) {
    double rji[3], rjk[3], rkl[3], rnj[3], rnk[3];
    for (int a = 0; a < 3; ++a) {
        rji[a] = S.x[3 * i + a] - S.x[3 * j + a];
        rjk[a] = S.x[3 * k + a] - S.x[3 * j + a];
        rkl[a] = S.x[3 * l + a] - S.x[3 * k + a];
    }
    rnj[0] = rji[1] * rjk[2] - rji[2] * rjk[1];
    rnj[1] = rji[2] * rjk[0] - rji[0] * rjk[2];
    rnj[2] = rji[0] * rjk[1] - rji[1] * rjk[0];
    rnk[0] = -rjk[1] * rkl[2] + rjk[2] * rkl[1];
    rnk[1] = -rjk[2] * rkl[0] + rjk[0] * rkl[2];
    rnk[2] = -rjk[0] * rkl[1] + rjk[1] * rkl[0];
    const double bj = sqrt(rnj[0] * rnj[0] + rnj[1] * rnj[1] + rnj[2] * rnj[2]);
    const double bk = sqrt(rnk[0] * rnk[0] + rnk[1] * rnk[1] + rnk[2] * rnk[2]);
    double scp = (rnj[0] * rnk[0] + rnj[1] * rnk[1] + rnj[2] * rnk[2]) / (bj * bk);
    scp = fmin(1.0, fmax(-1.0, scp));
    double phi = acos(scp);
    const double sgn = rjk[0] * (rnj[1] * rnk[2] - rnj[2] * rnk[1]) + rjk[1] * (rnj[2] * rnk[0] - rnj[0] * rnk[2]) +
                       rjk[2] * (rnj[0] * rnk[1] - rnj[1] * rnk[0]);
    if (sgn < 0) phi = -phi;
    double f1 = sin(phi);
    if (fabs(f1) < QREAL_EPS) f1 = QREAL_EPS;
    f1 = -1.0 / f1;
    double di[3], dl[3], rki[3], rlj[3];
    for (int a = 0; a < 3; ++a) {
        di[a] = f1 * (rnk[a] / (bj * bk) - scp * rnj[a] / (bj * bj));
        dl[a] = f1 * (rnj[a] / (bj * bk) - scp * rnk[a] / (bk * bk));
        rki[a] = rji[a] - rjk[a];
        rlj[a] = -rjk[a] - rkl[a];
    }
    dp[0] = rjk[1] * di[2] - rjk[2] * di[1];
    dp[1] = rjk[2] * di[0] - rjk[0] * di[2];
    dp[2] = rjk[0] * di[1] - rjk[1] * di[0];
    dp[3] = rki[1] * di[2] - rki[2] * di[1] + rkl[1] * dl[2] - rkl[2] * dl[1];
    dp[4] = rki[2] * di[0] - rki[0] * di[2] + rkl[2] * dl[0] - rkl[0] * dl[2];
    dp[5] = rki[0] * di[1] - rki[1] * di[0] + rkl[0] * dl[1] - rkl[1] * dl[0];
    dp[6] = rlj[1] * dl[2] - rlj[2] * dl[1] - rji[1] * di[2] + rji[2] * di[1];
    dp[7] = rlj[2] * dl[0] - rlj[0] * dl[2] - rji[2] * di[0] + rji[0] * di[2];
    dp[8] = rlj[0] * dl[1] - rlj[1] * dl[0] - rji[0] * di[1] + rji[1] * di[0];
    dp[9] = rjk[1] * dl[2] - rjk[2] * dl[1];
    dp[10] = rjk[2] * dl[0] - rjk[0] * dl[2];
    dp[11] = rjk[0] * dl[1] - rjk[1] * dl[0];
    return phi;
}
__device__ __forceinline__ void apply_dp(const DevSys &S, const int *at, double dv, const double dp[12]) {
    for (int n = 0; n < 4; ++n) grad_add(S, at[n], dv * dp[3 * n], dv * dp[3 * n + 1], dv * dp[3 * n + 2]);
}

// qbond/qangle/qtorsion/qimproper (src/md.f90:17022-17538) without EVB
// angle/torsion couplings.  One thread per (term, state).
__device__ void qbonded_block(const DevSys &S, int b) {
    const int id = b * blockDim.x + threadIdx.x;
    const int term = id / QG_MAXS, s = id % QG_MAXS;
    if (term >= S.nqt) return;
    const int traj = S.qt_traj[term];
    const TrajInfo &T = S.traj[traj];
    if (s >= T.nstates) return;
    const int ic = S.qt_cod[term * QG_MAXS + s];
    if (ic <= 0) return;
    const double *L = S.qt_lib + 4 * (ic - 1);
    const int *at = S.qt_atoms + 4 * term;
    const double lam = T.lambda[s];
    const int kind = S.qt_kind[term];
    double e = 0;
    int slot = EA_Q0 + EQ_N * s;
    const double pi = 3.14159265358979323846;
    if (kind == 0) {
        const int i = at[0], j = at[1];
        const double r0 = S.x[3 * j] - S.x[3 * i], r1 = S.x[3 * j + 1] - S.x[3 * i + 1], r2 = S.x[3 * j + 2] - S.x[3 * i + 2];
        const double b = sqrt(r0 * r0 + r1 * r1 + r2 * r2), db = b - L[2];
        const double fexp = exp(-L[1] * db);
        e = L[0] * (fexp * fexp - 2.0 * fexp) + 0.5 * L[3] * db * db;
        const double dv = (2.0 * L[0] * L[1] * (fexp - fexp * fexp) + L[3] * db) * lam / b;
        grad_add(S, j, r0 * dv, r1 * dv, r2 * dv);
        grad_add(S, i, -r0 * dv, -r1 * dv, -r2 * dv);
        slot += EQ_B;
    } else if (kind == 1) {
        double gi[3], gk[3];
        e = angle_grad(S, at[0], at[1], at[2], L[0], L[1], lam, gi, gk);
        grad_add(S, at[0], gi[0], gi[1], gi[2]);
        grad_add(S, at[2], gk[0], gk[1], gk[2]);
        grad_add(S, at[1], -(gi[0] + gk[0]), -(gi[1] + gk[1]), -(gi[2] + gk[2]));
        slot += EQ_A;
    } else if (kind == 2) {
        double dp[12];
        const double phi = dihedral(S, at[0], at[1], at[2], at[3], dp);
        const double arg = L[1] * phi - L[2];
        e = L[0] * (1.0 + cos(arg));
        apply_dp(S, at, -L[1] * L[0] * sin(arg) * lam, dp);
        slot += EQ_T;
    } else {
        double dp[12];
        const double phi = dihedral(S, at[0], at[1], at[2], at[3], dp);
        double arg = phi - L[1];
        arg = arg - 2.0 * pi * rint(arg / (2.0 * pi));
        const double dv = L[0] * arg;
        e = 0.5 * dv * arg;
        apply_dp(S, at, dv * lam, dp);
        slot += EQ_I;
    }
    fx_add(S.eacc + (size_t)traj * QG_NE + slot, e, S.status);
}

// bond/angle/torsion/improper(2), src/md.f90:1130-1405, 3130-3423,
// 17907-18054.  Terms are grouped per (trajectory, energy slot) and padded to
// whole blocks, so each block reduces into one slot.
__device__ void bonded_block(const DevSys &S, int b, double *red) {
    const int id = b * blockDim.x + threadIdx.x;
    const int traj = S.bt_blk_traj[b], slot = S.bt_blk_slot[b];
    const int c = S.bt_cod[id];
    double e = 0;
    const double pi = 3.14159265358979323846;
    if (c >= 0) {
        const int *at = S.bt_atoms + 4 * id;
        const double *L = S.bt_lib + 4 * c;
        const int kind = S.bt_kind[id];
        if (kind == 0) {
            const int i = at[0], j = at[1];
            const double r0 = S.x[3 * j] - S.x[3 * i], r1 = S.x[3 * j + 1] - S.x[3 * i + 1], r2 = S.x[3 * j + 2] - S.x[3 * i + 2];
            const double b = sqrt(r0 * r0 + r1 * r1 + r2 * r2), db = b - L[1];
            e = 0.5 * L[0] * db * db;
            const double dv = L[0] * db / b;
            grad_add(S, j, r0 * dv, r1 * dv, r2 * dv);
            grad_add(S, i, -r0 * dv, -r1 * dv, -r2 * dv);
        } else if (kind == 1) {
            double gi[3], gk[3];
            e = angle_grad(S, at[0], at[1], at[2], L[0], L[1], 1.0, gi, gk);
            grad_add(S, at[0], gi[0], gi[1], gi[2]);
            grad_add(S, at[2], gk[0], gk[1], gk[2]);
            grad_add(S, at[1], -(gi[0] + gk[0]), -(gi[1] + gk[1]), -(gi[2] + gk[2]));
        } else if (kind == 2) {
            double dp[12];
            const double phi = dihedral(S, at[0], at[1], at[2], at[3], dp);
            const double arg = L[1] * phi - L[2];
            e = L[0] * (1.0 + cos(arg)) * L[3];
            apply_dp(S, at, -L[1] * L[0] * sin(arg) * L[3], dp);
        } else if (kind == 3) {
            double dp[12];
            const double phi = dihedral(S, at[0], at[1], at[2], at[3], dp);
            double arg = phi - L[1];
            arg = arg - 2.0 * pi * rint(arg / (2.0 * pi));
            const double dv = L[0] * arg;
            e = 0.5 * dv * arg;
            apply_dp(S, at, dv, dp);
        } else {
            double dp[12];
            const double phi = dihedral(S, at[0], at[1], at[2], at[3], dp);
            const double arg = 2.0 * phi - L[1];
            e = L[0] * (1.0 + cos(arg));
            apply_dp(S, at, -2.0 * L[0] * sin(arg), dp);
        }
    }
    block_energy_d(S, traj, slot, e, red);
}

// fix_shell, src/md.f90:2816-2864 (no freeze).  One thread per solute atom.
__device__ void fix_shell_block(const DevSys &S, int b, const int *satom, double *red) {
    const int i = satom[b * blockDim.x + threadIdx.x];
    const int traj = i < 0 ? -1 - i : S.atraj[i];
    const TrajInfo &T = S.traj[traj];
    double efix = 0, eshell = 0;
    if (i >= 0 && (S.aexcl[i] || S.ashell[i])) {
        const double fk = S.aexcl[i] ? T.fk_fix : T.fk_pshell;
        const double d0 = S.x[3 * i] - S.xtop[3 * i], d1 = S.x[3 * i + 1] - S.xtop[3 * i + 1], d2 = S.x[3 * i + 2] - S.xtop[3 * i + 2];
        const double e = 0.5 * fk * (d0 * d0 + d1 * d1 + d2 * d2);
        if (S.aexcl[i]) efix = e;
        if (S.ashell[i]) eshell = e;
        grad_add(S, i, fk * d0, fk * d1, fk * d2);
    }
    block_energy_d(S, traj, EA_RST_FIX, efix, red);
    block_energy_d(S, traj, EA_RST_SHELL, eshell, red);
}

// restrain_solvent, src/md.f90:18055-18102.  One thread per water.
__device__ void restrain_solvent_block(const DevSys &S, int b, const int *wgrp, double *red) {
    const int w = wgrp[b * blockDim.x + threadIdx.x];
    const int traj = w < 0 ? -1 - w : S.g_traj[w];
    const TrajInfo &T = S.traj[traj];
    double erst = 0;
    if (w >= 0) {
        const int i = S.g_switch[w];
        if (!S.aexcl[i]) {
            const double Tfree = S.tstate[traj].Tfree;
            const double shift = T.fk_wsphere != 0.0 ? sqrt(BOLTZ * Tfree / T.fk_wsphere) : 0.0;
            const double d0 = S.x[3 * i] - T.xwcent[0], d1 = S.x[3 * i + 1] - T.xwcent[1], d2 = S.x[3 * i + 2] - T.xwcent[2];
            const double b = sqrt(d0 * d0 + d1 * d1 + d2 * d2);
            const double db = b - (T.rwat - shift);
            double dv;
            if (db > 0) {
                erst = 0.5 * T.fk_wsphere * db * db - T.Dwmz;
                dv = T.fk_wsphere * db / b;
            } else if (b > 0.0) {
                const double fexp = exp(T.awmz * db);
                erst = T.Dwmz * (fexp * fexp - 2.0 * fexp);
                dv = -2.0 * T.Dwmz * T.awmz * (fexp - fexp * fexp) / b;
            } else { dv = 0; erst = 0; }
            grad_add(S, i, dv * d0, dv * d1, dv * d2);
        }
    }
    block_energy_d(S, traj, EA_RST_RAD, erst, red);
}

// offdiag, src/md.f90:15444-15470: Hij = A exp(-mu r_kl).
__device__ void offdiag_block(const DevSys &S, int blk) {
    const int k = blk * blockDim.x + threadIdx.x;
    if (k >= S.nod) return;
    const int traj = S.od_traj[k];
    const int a = S.q_atom[S.od_kl[2 * k]], b = S.q_atom[S.od_kl[2 * k + 1]];
    const double d0 = S.x[3 * b] - S.x[3 * a], d1 = S.x[3 * b + 1] - S.x[3 * a + 1], d2 = S.x[3 * b + 2] - S.x[3 * a + 2];
    const double r = sqrt(d0 * d0 + d1 * d1 + d2 * d2);
    const int slot = S.od_ij[2 * k];   // index of the coupling within its trajectory
    double *o = S.od_out + ((size_t)traj * QG_MAXOD + slot) * 2;
    o[0] = S.od_Amu[2 * k] * exp(-S.od_Amu[2 * k + 1] * r);
    o[1] = r;
}

// The small terms share one launch: consecutive block ranges select the term.
struct MiscPlan {
    int nqq, nbt, nfix, nrad, nqb, nod;    // blocks per term
};

__global__ void __launch_bounds__(QG_BLOCK) k_misc(DevSys S, MiscPlan P, const int *qq_traj, const int *qq_s,
                                                   const int *satom, const int *wgrp) {
    __shared__ double red[QG_BLOCK / 32];
    int b = blockIdx.x;
    if (b < P.nqq) { qq_block(S, b, qq_traj, qq_s, red); return; }
    b -= P.nqq;
    if (b < P.nbt) { bonded_block(S, b, red); return; }
    b -= P.nbt;
    if (b < P.nfix) { fix_shell_block(S, b, satom, red); return; }
    b -= P.nfix;
    if (b < P.nrad) { restrain_solvent_block(S, b, wgrp, red); return; }
    b -= P.nrad;
    if (b < P.nqb) { qbonded_block(S, b); return; }
    b -= P.nqb;
    if (b < P.nod) { offdiag_block(S, b); return; }
}

static inline int nblk(int n, int b) { return (n + b - 1) / b; }

void launch_misc(const DevSys &S, const BlockTables &B, LaunchCtx &L, int terms) {
    MiscPlan P{};
    P.nqq = (terms & QGPU_TERMS_QQ) ? B.nqqblk : 0;
    P.nbt = (terms & QGPU_TERMS_BONDED) ? S.nbt / QG_BLOCK : 0;
    P.nfix = (terms & QGPU_TERMS_RESTRAINT) ? B.nsatom / QG_BLOCK : 0;
    P.nrad = (terms & QGPU_TERMS_RESTRAINT) ? B.nwgrp / QG_BLOCK : 0;
    P.nqb = (terms & QGPU_TERMS_QBONDED) ? nblk(S.nqt * QG_MAXS, QG_BLOCK) : 0;
    P.nod = nblk(S.nod, QG_BLOCK);
    const int nb = P.nqq + P.nbt + P.nfix + P.nrad + P.nqb + P.nod;
    if (!nb) return;
    prof_begin(L, "k_misc");
    k_misc<<<nb, QG_BLOCK, 0, L.stream>>>(S, P, B.qqblk_traj, B.qqblk_s, B.satom, B.wgrp);
    prof_end(L);
    (*L.nlaunch)++;
}
