// k_small.cu -- the small terms of pot_energy (src/md.f90:16100-16150):
// nonbond_qq, the per-state Q bonded terms, classical bonded terms, the sphere
// restraints and the EVB off-diagonal couplings.  These are O(Q^2) or O(N)
// with little arithmetic.  Each term is written once over a real type R:
//   R = double on the steps whose energies are recorded and in the drop-in
//          qgpu_forces call (coordinates from the FP64 x, FP64 parameters);
//   R = float on every other MD step (relative vectors from the hi/lo float
//          coordinates, float parameter copies), because GB300 issues FP64 at
//          1/64 of the FP32 rate and these terms run every step.
#include <math.h>

#include "qgpu_internal.cuh"

#define QREAL_EPS 1.0e-14   // src/sizes.f90:48

template <typename R>
struct V3 {
    R x, y, z;
};

// b - a from the coordinates of the precision in use
template <typename R>
__device__ __forceinline__ V3<R> rel(const DevSys &S, int a, int b);
template <>
__device__ __forceinline__ V3<double> rel<double>(const DevSys &S, int a, int b) {
    return {S.x[3 * b] - S.x[3 * a], S.x[3 * b + 1] - S.x[3 * a + 1], S.x[3 * b + 2] - S.x[3 * a + 2]};
}
template <>
__device__ __forceinline__ V3<float> rel<float>(const DevSys &S, int a, int b) {
    const float3 d = dpos(S.pos[a], S.poslo[a], S.pos[b], S.poslo[b]);
    return {d.x, d.y, d.z};
}

// parameter access per precision
template <typename R> struct P;
template <>
struct P<double> {
    static __device__ __forceinline__ double crg(const DevSys &S, int i) { return S.crg_d[i]; }
    static __device__ __forceinline__ double qcrg(const DevSys &S, int k) { return S.qcrg_d[k]; }
    static __device__ __forceinline__ double avdw(const DevSys &S, int k) { return S.avdw_d[k]; }
    static __device__ __forceinline__ double bvdw(const DevSys &S, int k) { return S.bvdw_d[k]; }
    static __device__ __forceinline__ double qavdw(const DevSys &S, int k) { return S.qavdw_d[k]; }
    static __device__ __forceinline__ double qbvdw(const DevSys &S, int k) { return S.qbvdw_d[k]; }
    static __device__ __forceinline__ double sc(const DevSys &S, size_t k) { return S.sc_d[k]; }
    static __device__ __forceinline__ double qq_els(const DevSys &S, int k) { return S.qq_els[k]; }
    static __device__ __forceinline__ const double *qt_lib(const DevSys &S) { return S.qt_lib; }
    static __device__ __forceinline__ const double *bt_lib(const DevSys &S) { return S.bt_lib; }
    static __device__ __forceinline__ double lambda(const TrajInfo &T, int s) { return T.lambda[s]; }
    static __device__ __forceinline__ double el14(const TrajInfo &T) { return T.el14d; }
    static __device__ __forceinline__ void grad(const DevSys &S, int a, double gx, double gy, double gz) {
        fx_add(S.fx + 3 * a, gx, S.status);
        fx_add(S.fx + 3 * a + 1, gy, S.status);
        fx_add(S.fx + 3 * a + 2, gz, S.status);
    }
    static __device__ __forceinline__ long long fx(double v, int *st) { return d2fx_chk(v, st); }
};
template <>
struct P<float> {
    static __device__ __forceinline__ float crg(const DevSys &S, int i) { return S.pos[i].w; }
    static __device__ __forceinline__ float qcrg(const DevSys &S, int k) { return S.qcrg_f[k]; }
    static __device__ __forceinline__ float avdw(const DevSys &S, int k) { return S.avdw[k]; }
    static __device__ __forceinline__ float bvdw(const DevSys &S, int k) { return S.bvdw[k]; }
    static __device__ __forceinline__ float qavdw(const DevSys &S, int k) { return S.qavdw[k]; }
    static __device__ __forceinline__ float qbvdw(const DevSys &S, int k) { return S.qbvdw[k]; }
    static __device__ __forceinline__ float sc(const DevSys &S, size_t k) { return S.sc_f[k]; }
    static __device__ __forceinline__ float qq_els(const DevSys &S, int k) { return S.qq_elsf[k]; }
    static __device__ __forceinline__ const float *qt_lib(const DevSys &S) { return S.qt_libf; }
    static __device__ __forceinline__ const float *bt_lib(const DevSys &S) { return S.bt_libf; }
    static __device__ __forceinline__ float lambda(const TrajInfo &T, int s) { return T.lambdaf[s]; }
    static __device__ __forceinline__ float el14(const TrajInfo &T) { return T.el14; }
    static __device__ __forceinline__ void grad(const DevSys &S, int a, float gx, float gy, float gz) {
        fx_addf(S.fx + 3 * a, gx, S.status);
        fx_addf(S.fx + 3 * a + 1, gy, S.status);
        fx_addf(S.fx + 3 * a + 2, gz, S.status);
    }
    static __device__ __forceinline__ long long fx(float v, int *st) { return f2fx_chk(v, st); }
};

typedef long long Red[4][QG_BLOCK / 32];

// nonbond_qq, src/md.f90:13491-13636.  One block per (trajectory, state).
template <typename R>
__device__ void qq_block(const DevSys &S, int b, const int *blk_traj, const int *blk_s, Red &red) {
    typedef P<R> p;
    const int traj = blk_traj[b], s = blk_s[b];
    const TrajInfo &T = S.traj[traj];
    const R lam = p::lambda(T, s);
    const int ntq = T.natyps + T.nqat;
    R eqq_el = 0, eqq_vdw = 0, eqp_el = 0, eqp_vdw = 0;
    for (int k = T.qq0[s] + threadIdx.x; k < T.qq0[s] + T.nqq[s]; k += blockDim.x) {
        const int q = S.qq_iq[k], i = S.q_atom[q], j = S.qq_j[k], jq = S.qq_jq[k], c = S.qq_lj[k];
        const int iql = q - T.q0;
        const R qi = p::qcrg(S, q * QG_MAXS + s);
        R qj, aLJ, bLJ;
        if (T.arith) {
            // nonbon2_qq (src/md.f90:11780-11998): a parameters summed (the
            // exponential Q-Q repulsion of code 2 multiplies them), b multiplied
            if (!T.qvdw) {
                const int ti = S.atype[i], tj = S.atype[j];
                aLJ = p::avdw(S, ti * 3 + c - 1) + p::avdw(S, tj * 3 + c - 1);
                bLJ = p::bvdw(S, ti * 3 + c - 1) * p::bvdw(S, tj * 3 + c - 1);
                qj = jq >= 0 ? p::qcrg(S, jq * QG_MAXS + s) : p::crg(S, j);
            } else {
                const int ti = S.qiac[q * QG_MAXS + s];
                aLJ = p::qavdw(S, ti * 3 + c - 1);
                bLJ = p::qbvdw(S, ti * 3 + c - 1);
                if (jq >= 0) {
                    const int tj = S.qiac[jq * QG_MAXS + s];
                    if (c == 2) aLJ = aLJ * p::qavdw(S, tj * 3 + c - 1);
                    else aLJ = aLJ + p::qavdw(S, tj * 3 + c - 1);
                    bLJ = bLJ * p::qbvdw(S, tj * 3 + c - 1);
                    qj = p::qcrg(S, jq * QG_MAXS + s);
                } else {
                    if (c == 2) { aLJ = p::qavdw(S, ti * 3); bLJ = p::qbvdw(S, ti * 3); }
                    const int tj = S.atype[j];
                    aLJ = aLJ + p::avdw(S, tj * 3 + c - 1);
                    bLJ = bLJ * p::bvdw(S, tj * 3 + c - 1);
                    qj = p::crg(S, j);
                }
            }
        } else if (!T.qvdw) {
            const int ti = S.atype[i], tj = S.atype[j];
            aLJ = p::avdw(S, ti * 3 + c - 1) * p::avdw(S, tj * 3 + c - 1);
            bLJ = p::bvdw(S, ti * 3 + c - 1) * p::bvdw(S, tj * 3 + c - 1);
            qj = jq >= 0 ? p::qcrg(S, jq * QG_MAXS + s) : p::crg(S, j);
        } else {
            const int ti = S.qiac[q * QG_MAXS + s];
            aLJ = p::qavdw(S, ti * 3 + c - 1);
            bLJ = p::qbvdw(S, ti * 3 + c - 1);
            if (jq >= 0) {
                const int tj = S.qiac[jq * QG_MAXS + s];
                aLJ *= p::qavdw(S, tj * 3 + c - 1);
                bLJ *= p::qbvdw(S, tj * 3 + c - 1);
                qj = p::qcrg(S, jq * QG_MAXS + s);
            } else {
                if (c == 2) { aLJ = p::qavdw(S, ti * 3); bLJ = p::qbvdw(S, ti * 3); }
                const int tj = S.atype[j];
                aLJ *= p::avdw(S, tj * 3 + c - 1);
                bLJ *= p::bvdw(S, tj * 3 + c - 1);
                qj = p::crg(S, j);
            }
        }
        const V3<R> d = rel<R>(S, i, j);
        R r2 = d.x * d.x + d.y * d.y + d.z * d.z;
        const R r6hc = r2 * r2 * r2;
        // softcore column natyps+jq, natyps for a non-Q partner (src/md.f90:13561)
        const int col = jq >= 0 ? T.natyps + (jq - T.q0) : T.natyps - 1;
        R r6 = r6hc + p::sc(S, (size_t)T.sc0 + ((size_t)iql * ntq + col) * QG_MAXS + s);
        r6 = R(1) / r6;
        const R r12 = r6 * r6;
        r2 = R(1) / r2;
        const R r = sqrt(r2);
        R Vel = qi * qj * r * p::qq_els(S, k);
        if (c == 3) Vel *= p::el14(T);
        R Va, Vb, dv;
        if (T.qvdw && jq >= 0 && c == 2) {
            Va = aLJ * exp(-bLJ / r);
            Vb = 0;
            dv = r2 * (-Vel - bLJ * Va / r) * lam;
        } else if (T.arith) {
            R a6 = aLJ * aLJ;
            a6 = a6 * a6 * a6;
            Va = bLJ * a6 * a6 * r12;
            Vb = R(2) * bLJ * a6 * r6;
            dv = r2 * (-Vel - (R(12) * Va - R(6) * Vb) * r6 * r6hc) * lam;
        } else {
            Va = aLJ * r12;
            Vb = bLJ * r6;
            dv = r2 * (-Vel - (R(12) * Va - R(6) * Vb) * r6hc * r6) * lam;
        }
        p::grad(S, i, -dv * d.x, -dv * d.y, -dv * d.z);
        p::grad(S, j, dv * d.x, dv * d.y, dv * d.z);
        if (jq >= 0) { eqq_el += Vel; eqq_vdw += Va - Vb; }
        else { eqp_el += Vel; eqp_vdw += Va - Vb; }
    }
    const int base = EA_Q0 + EQ_N * s;
    const int slots[4] = {base + EQ_QQ_EL, base + EQ_QQ_VDW, base + EQ_QP_EL, base + EQ_QP_VDW};
    long long v[4] = {p::fx(eqq_el, S.status), p::fx(eqq_vdw, S.status), p::fx(eqp_el, S.status),
                      p::fx(eqp_vdw, S.status)};
    block_energies_fx<4>(S.eacc + (size_t)traj * QG_NE, slots, v, red);
}

// --------------------------------------------------- angle / dihedral
template <typename R>
__device__ R angle_grad(const DevSys &S, int i, int j, int k, R fk, R ang0, R scale, R gi[3], R gk[3]) {
    const V3<R> a = rel<R>(S, j, i), c = rel<R>(S, j, k);   // rji, rjk
    const R rji[3] = {a.x, a.y, a.z}, rjk[3] = {c.x, c.y, c.z};
    const R bji = sqrt(rji[0] * rji[0] + rji[1] * rji[1] + rji[2] * rji[2]);
    const R bjk = sqrt(rjk[0] * rjk[0] + rjk[1] * rjk[1] + rjk[2] * rjk[2]);
    R scp = (rji[0] * rjk[0] + rji[1] * rjk[1] + rji[2] * rjk[2]) / (bji * bjk);
    scp = fmin(R(1), fmax(R(-1), scp));
    const R ang = acos(scp), da = ang - ang0;
    const R dv = fk * da * scale;
    R f1 = sin(ang);
    if (fabs(f1) < R(QREAL_EPS)) f1 = R(QREAL_EPS);
    f1 = R(-1) / f1;
    for (int q = 0; q < 3; ++q) {
        gi[q] = dv * f1 * (rjk[q] / (bji * bjk) - scp * rji[q] / (bji * bji));
        gk[q] = dv * f1 * (rji[q] / (bji * bjk) - scp * rjk[q] / (bjk * bjk));
    }
    return R(0.5) * fk * da * da;
}

// dihedral angle and its derivative components (src/md.f90:17241-17538)
template <typename R>
__device__ R dihedral(const DevSys &S, int i, int j, int k, int l, R dp[12]) {
    const V3<R> a = rel<R>(S, j, i), b = rel<R>(S, j, k), c = rel<R>(S, k, l);
    const R rji[3] = {a.x, a.y, a.z}, rjk[3] = {b.x, b.y, b.z}, rkl[3] = {c.x, c.y, c.z};
    R rnj[3], rnk[3];
    rnj[0] = rji[1] * rjk[2] - rji[2] * rjk[1];
    rnj[1] = rji[2] * rjk[0] - rji[0] * rjk[2];
    rnj[2] = rji[0] * rjk[1] - rji[1] * rjk[0];
    rnk[0] = -rjk[1] * rkl[2] + rjk[2] * rkl[1];
    rnk[1] = -rjk[2] * rkl[0] + rjk[0] * rkl[2];
    rnk[2] = -rjk[0] * rkl[1] + rjk[1] * rkl[0];
    const R bj = sqrt(rnj[0] * rnj[0] + rnj[1] * rnj[1] + rnj[2] * rnj[2]);
    const R bk = sqrt(rnk[0] * rnk[0] + rnk[1] * rnk[1] + rnk[2] * rnk[2]);
    R scp = (rnj[0] * rnk[0] + rnj[1] * rnk[1] + rnj[2] * rnk[2]) / (bj * bk);
    scp = fmin(R(1), fmax(R(-1), scp));
    R phi = acos(scp);
    const R sgn = rjk[0] * (rnj[1] * rnk[2] - rnj[2] * rnk[1]) + rjk[1] * (rnj[2] * rnk[0] - rnj[0] * rnk[2]) +
                  rjk[2] * (rnj[0] * rnk[1] - rnj[1] * rnk[0]);
    if (sgn < 0) phi = -phi;
    R f1 = sin(phi);
    if (fabs(f1) < R(QREAL_EPS)) f1 = R(QREAL_EPS);
    f1 = R(-1) / f1;
    R di[3], dl[3], rki[3], rlj[3];
    for (int q = 0; q < 3; ++q) {
        di[q] = f1 * (rnk[q] / (bj * bk) - scp * rnj[q] / (bj * bj));
        dl[q] = f1 * (rnj[q] / (bj * bk) - scp * rnk[q] / (bk * bk));
        rki[q] = rji[q] - rjk[q];
        rlj[q] = -rjk[q] - rkl[q];
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
// FP32 forms of the two above.  The reference's expressions divide by
// sin(angle) after cancelling terms of size 1 (the component of one normal
// along the other), which in FP32 loses every digit for planar torsions and
// impropers.  The float path takes the same angles from atan2 (the same
// value and sign convention: phi < 0 when rjk.(rnj x rnk) < 0) and the
// dihedral gradient in the cancellation-free form of Blondel & Karplus,
// J. Comput. Chem. 17, 1132 (1996): with b1 = rji, b2 = rjk, b3 = rkl,
// m = b1 x b2, n = b3 x b2,
//   dphi/dri = |b2|/|m|^2 m,   dphi/drl = -|b2|/|n|^2 n,
//   dphi/drj = -gi + (b1.b2/|b2|^2) gi + (b3.b2/|b2|^2) gl,
//   dphi/drk = -gl - (b1.b2/|b2|^2) gi - (b3.b2/|b2|^2) gl.
template <>
__device__ float angle_grad<float>(const DevSys &S, int i, int j, int k, float fk, float ang0, float scale, float gi[3],
                                   float gk[3]) {
    const V3<float> a = rel<float>(S, j, i), c = rel<float>(S, j, k);
    const float bji = sqrtf(a.x * a.x + a.y * a.y + a.z * a.z), bjk = sqrtf(c.x * c.x + c.y * c.y + c.z * c.z);
    const float cx = a.y * c.z - a.z * c.y, cy = a.z * c.x - a.x * c.z, cz = a.x * c.y - a.y * c.x;
    const float sn = sqrtf(cx * cx + cy * cy + cz * cz), cs = a.x * c.x + a.y * c.y + a.z * c.z;
    const float ang = atan2f(sn, cs), da = ang - ang0;
    const float inv = 1.f / (bji * bjk);
    const float scp = cs * inv;
    float f1 = sn * inv;
    if (f1 < (float)QREAL_EPS) f1 = (float)QREAL_EPS;
    const float dvf = -fk * da * scale / f1;
    const float rji[3] = {a.x, a.y, a.z}, rjk[3] = {c.x, c.y, c.z};
    for (int q = 0; q < 3; ++q) {
        gi[q] = dvf * (rjk[q] * inv - scp * rji[q] / (bji * bji));
        gk[q] = dvf * (rji[q] * inv - scp * rjk[q] / (bjk * bjk));
    }
    return 0.5f * fk * da * da;
}
template <>
__device__ float dihedral<float>(const DevSys &S, int i, int j, int k, int l, float dp[12]) {
    const V3<float> b1 = rel<float>(S, j, i), b2 = rel<float>(S, j, k), b3 = rel<float>(S, k, l);
    const float mx = b1.y * b2.z - b1.z * b2.y, my = b1.z * b2.x - b1.x * b2.z, mz = b1.x * b2.y - b1.y * b2.x;
    const float nx = b3.y * b2.z - b3.z * b2.y, ny = b3.z * b2.x - b3.x * b2.z, nz = b3.x * b2.y - b3.y * b2.x;
    const float mm = mx * mx + my * my + mz * mz, nn = nx * nx + ny * ny + nz * nz;
    const float b22 = b2.x * b2.x + b2.y * b2.y + b2.z * b2.z, b2n = sqrtf(b22);
    const float c = mx * nx + my * ny + mz * nz;
    const float s = (b2.x * (my * nz - mz * ny) + b2.y * (mz * nx - mx * nz) + b2.z * (mx * ny - my * nx)) / b2n;
    const float phi = atan2f(s, c);
    const float fi = b2n / mm, fl = -b2n / nn;
    const float gi[3] = {fi * mx, fi * my, fi * mz}, gl[3] = {fl * nx, fl * ny, fl * nz};
    const float P = (b1.x * b2.x + b1.y * b2.y + b1.z * b2.z) / b22;
    const float Q = (b3.x * b2.x + b3.y * b2.y + b3.z * b2.z) / b22;
    for (int q = 0; q < 3; ++q) {
        dp[q] = gi[q];
        dp[3 + q] = -gi[q] + P * gi[q] + Q * gl[q];
        dp[6 + q] = -gl[q] - P * gi[q] - Q * gl[q];
        dp[9 + q] = gl[q];
    }
    return phi;
}

template <typename R>
__device__ __forceinline__ void apply_dp(const DevSys &S, const int *at, R dv, const R dp[12]) {
    for (int n = 0; n < 4; ++n) P<R>::grad(S, at[n], dv * dp[3 * n], dv * dp[3 * n + 1], dv * dp[3 * n + 2]);
}

// qbond/qangle/qtorsion/qimproper (src/md.f90:17022-17538) without EVB
// angle/torsion couplings.  One thread per (term, state).
template <typename R>
__device__ void qbonded_block(const DevSys &S, int b, int qt0, int nqt) {
    typedef P<R> p;
    const int id = b * blockDim.x + threadIdx.x;
    const int s = id % QG_MAXS;
    if (id / QG_MAXS >= nqt) return;
    const int term = qt0 + id / QG_MAXS;
    const int traj = S.qt_traj[term];
    const TrajInfo &T = S.traj[traj];
    if (s >= T.nstates) return;
    const int ic = S.qt_cod[term * QG_MAXS + s];
    if (ic <= 0) return;
    const auto *L = p::qt_lib(S) + 4 * (ic - 1);
    const int *at = S.qt_atoms + 4 * term;
    const R lam = p::lambda(T, s);
    const int kind = S.qt_kind[term];
    R e = 0;
    int slot = EA_Q0 + EQ_N * s;
    const R pi = R(3.14159265358979323846);
    if (kind == 0) {
        const int i = at[0], j = at[1];
        const V3<R> r = rel<R>(S, i, j);
        const R bl = sqrt(r.x * r.x + r.y * r.y + r.z * r.z), db = bl - L[2];
        const R fexp = exp(-L[1] * db);
        e = L[0] * (fexp * fexp - R(2) * fexp) + R(0.5) * L[3] * db * db;
        const R dv = (R(2) * L[0] * L[1] * (fexp - fexp * fexp) + L[3] * db) * lam / bl;
        p::grad(S, j, r.x * dv, r.y * dv, r.z * dv);
        p::grad(S, i, -r.x * dv, -r.y * dv, -r.z * dv);
        slot += EQ_B;
    } else if (kind == 1) {
        R gi[3], gk[3];
        e = angle_grad<R>(S, at[0], at[1], at[2], L[0], L[1], lam, gi, gk);
        p::grad(S, at[0], gi[0], gi[1], gi[2]);
        p::grad(S, at[2], gk[0], gk[1], gk[2]);
        p::grad(S, at[1], -(gi[0] + gk[0]), -(gi[1] + gk[1]), -(gi[2] + gk[2]));
        slot += EQ_A;
    } else if (kind == 2) {
        R dp[12];
        const R phi = dihedral<R>(S, at[0], at[1], at[2], at[3], dp);
        const R arg = L[1] * phi - L[2];
        e = L[0] * (R(1) + cos(arg));
        apply_dp<R>(S, at, -L[1] * L[0] * sin(arg) * lam, dp);
        slot += EQ_T;
    } else {
        R dp[12];
        const R phi = dihedral<R>(S, at[0], at[1], at[2], at[3], dp);
        R arg = phi - L[1];
        arg = arg - R(2) * pi * rint(arg / (R(2) * pi));
        const R dv = L[0] * arg;
        e = R(0.5) * dv * arg;
        apply_dp<R>(S, at, dv * lam, dp);
        slot += EQ_I;
    }
    const long long q = p::fx(e, S.status);
    if (q) atomicAdd(S.eacc + (size_t)traj * QG_NE + slot, (unsigned long long)q);
}

// bond/angle/torsion/improper(2), src/md.f90:1130-1405, 3130-3423,
// 17907-18054.  Terms are grouped per (trajectory, energy slot) and padded to
// whole blocks, so each block reduces into one slot.
template <typename R>
__device__ void bonded_block(const DevSys &S, int b, Red &red) {
    typedef P<R> p;
    const int id = b * blockDim.x + threadIdx.x;
    const int traj = S.bt_blk_traj[b];
    const int c = S.bt_cod[id];
    R e = 0;
    const R pi = R(3.14159265358979323846);
    if (c >= 0) {
        const int *at = S.bt_atoms + 4 * id;
        const auto *L = p::bt_lib(S) + 4 * c;
        const int kind = S.bt_kind[id];
        if (kind == 0) {
            const int i = at[0], j = at[1];
            const V3<R> r = rel<R>(S, i, j);
            const R bl = sqrt(r.x * r.x + r.y * r.y + r.z * r.z), db = bl - L[1];
            e = R(0.5) * L[0] * db * db;
            const R dv = L[0] * db / bl;
            p::grad(S, j, r.x * dv, r.y * dv, r.z * dv);
            p::grad(S, i, -r.x * dv, -r.y * dv, -r.z * dv);
        } else if (kind == 1) {
            R gi[3], gk[3];
            e = angle_grad<R>(S, at[0], at[1], at[2], L[0], L[1], R(1), gi, gk);
            p::grad(S, at[0], gi[0], gi[1], gi[2]);
            p::grad(S, at[2], gk[0], gk[1], gk[2]);
            p::grad(S, at[1], -(gi[0] + gk[0]), -(gi[1] + gk[1]), -(gi[2] + gk[2]));
        } else if (kind == 2) {
            R dp[12];
            const R phi = dihedral<R>(S, at[0], at[1], at[2], at[3], dp);
            const R arg = L[1] * phi - L[2];
            e = L[0] * (R(1) + cos(arg)) * L[3];
            apply_dp<R>(S, at, -L[1] * L[0] * sin(arg) * L[3], dp);
        } else if (kind == 3) {
            R dp[12];
            const R phi = dihedral<R>(S, at[0], at[1], at[2], at[3], dp);
            R arg = phi - L[1];
            arg = arg - R(2) * pi * rint(arg / (R(2) * pi));
            const R dv = L[0] * arg;
            e = R(0.5) * dv * arg;
            apply_dp<R>(S, at, dv, dp);
        } else {
            R dp[12];
            const R phi = dihedral<R>(S, at[0], at[1], at[2], at[3], dp);
            const R arg = R(2) * phi - L[1];
            e = L[0] * (R(1) + cos(arg));
            apply_dp<R>(S, at, R(-2) * L[0] * sin(arg), dp);
        }
    }
    const int slots[1] = {S.bt_blk_slot[b]};
    long long v[1] = {p::fx(e, S.status)};
    block_energies_fx<1>(S.eacc + (size_t)traj * QG_NE, slots, v, red);
}

// fix_shell, src/md.f90:2816-2864 (no freeze).  One thread per solute atom.
template <typename R>
__device__ void fix_shell_block(const DevSys &S, int b, const int *satom, Red &red) {
    typedef P<R> p;
    const int i = satom[b * blockDim.x + threadIdx.x];
    const int traj = i < 0 ? -1 - i : S.atraj[i];
    const TrajInfo &T = S.traj[traj];
    R efix = 0, eshell = 0;
    // sphere only (pot_energy :16114-16116)
    if (i >= 0 && !T.pbc && (S.aexcl[i] || S.ashell[i])) {
        R fk, d0, d1, d2;
        if (sizeof(R) == 8) {
            fk = S.aexcl[i] ? R(T.fk_fix) : R(T.fk_pshell);
            d0 = R(S.x[3 * i] - S.xtop[3 * i]); d1 = R(S.x[3 * i + 1] - S.xtop[3 * i + 1]);
            d2 = R(S.x[3 * i + 2] - S.xtop[3 * i + 2]);
        } else {
            fk = S.aexcl[i] ? R(T.fk_fixf) : R(T.fk_pshellf);
            const float3 d = dpos(S.xtoph[i], S.xtopl[i], S.pos[i], S.poslo[i]);
            d0 = R(d.x); d1 = R(d.y); d2 = R(d.z);
        }
        const R e = R(0.5) * fk * (d0 * d0 + d1 * d1 + d2 * d2);
        if (S.aexcl[i]) efix = e;
        if (S.ashell[i]) eshell = e;
        p::grad(S, i, fk * d0, fk * d1, fk * d2);
    }
    const int slots[2] = {EA_RST_FIX, EA_RST_SHELL};
    long long v[2] = {p::fx(efix, S.status), p::fx(eshell, S.status)};
    block_energies_fx<2>(S.eacc + (size_t)traj * QG_NE, slots, v, red);
}

// restrain_solvent, src/md.f90:18055-18102.  One thread per water.  The shift
// sqrt(Boltz*Tfree/fk_wsphere) is formed by k_finalize with the temperature.
template <typename R>
__device__ void restrain_solvent_block(const DevSys &S, int b, const int *wgrp, Red &red) {
    typedef P<R> p;
    const int w = wgrp[b * blockDim.x + threadIdx.x];
    const int traj = w < 0 ? -1 - w : S.g_traj[w];
    const TrajInfo &T = S.traj[traj];
    R erst = 0;
    // sphere only (pot_energy :16120-16124)
    if (w >= 0 && !T.pbc) {
        const int i = S.g_switch[w];
        if (!S.aexcl[i]) {
            R d0, d1, d2, fk, rwat, Dwmz, awmz, shift;
            if (sizeof(R) == 8) {
                d0 = R(S.x[3 * i] - T.xwcent[0]); d1 = R(S.x[3 * i + 1] - T.xwcent[1]);
                d2 = R(S.x[3 * i + 2] - T.xwcent[2]);
                fk = R(T.fk_wsphere); rwat = R(T.rwat); Dwmz = R(T.Dwmz); awmz = R(T.awmz);
                shift = R(S.tstate[traj].wshiftf);
            } else {
                // the float coordinates are relative to the origin, which is xwcent
                const float4 h = S.pos[i], l = S.poslo[i];
                d0 = R(h.x + l.x); d1 = R(h.y + l.y); d2 = R(h.z + l.z);
                fk = R(T.fk_wspheref); rwat = R(T.rwatf); Dwmz = R(T.Dwmzf); awmz = R(T.awmzf);
                shift = R(S.tstate[traj].wshiftf);
            }
            const R bl = sqrt(d0 * d0 + d1 * d1 + d2 * d2);
            const R db = bl - (rwat - shift);
            R dv;
            if (db > 0) {
                erst = R(0.5) * fk * db * db - Dwmz;
                dv = fk * db / bl;
            } else if (bl > R(0)) {
                const R fexp = exp(awmz * db);
                erst = Dwmz * (fexp * fexp - R(2) * fexp);
                dv = R(-2) * Dwmz * awmz * (fexp - fexp * fexp) / bl;
            } else { dv = 0; erst = 0; }
            p::grad(S, i, dv * d0, dv * d1, dv * d2);
        }
    }
    const int slots[1] = {EA_RST_RAD};
    long long v[1] = {p::fx(erst, S.status)};
    block_energies_fx<1>(S.eacc + (size_t)traj * QG_NE, slots, v, red);
}

// p_restrain's sequence restraints, src/md.f90:15484-15576.  One block per
// restraint; an atom of the range takes part when heavy, or when the H flag
// is set and it is not a frozen excluded atom.  to_centre 1 / 2 restrain the
// (mass-weighted) mean displacement from the topology and apply fk*dr
// (x mass/12.010 for the geometric centre) to every taking part atom;
// to_centre 0 restrains each atom.
template <typename R>
__device__ void seqrst_block(const DevSys &S, int b, Red &red) {
    typedef P<R> p;
    __shared__ R sw[4][QG_BLOCK / 32];
    __shared__ R tot[4];
    const int i0 = S.rs_i0[b], i1 = S.rs_i1[b], ih = S.rs_ih[b], tc = S.rs_tc[b], traj = S.rs_traj[b];
    const TrajInfo &T = S.traj[traj];
    const R fk = R(S.rs_fk[b]);
    auto sel = [&](int i) { return S.aheavy[i] || (ih == 1 && !(S.aexcl[i] && T.freeze)); };
    auto disp = [&](int i, R &d0, R &d1, R &d2) {
        if (sizeof(R) == 8) {
            d0 = R(S.x[3 * i] - S.xtop[3 * i]); d1 = R(S.x[3 * i + 1] - S.xtop[3 * i + 1]);
            d2 = R(S.x[3 * i + 2] - S.xtop[3 * i + 2]);
        } else {
            const float3 d = dpos(S.xtoph[i], S.xtopl[i], S.pos[i], S.poslo[i]);
            d0 = R(d.x); d1 = R(d.y); d2 = R(d.z);
        }
    };
    R e = 0;
    if (tc == 1 || tc == 2) {
        R acc[4] = {0, 0, 0, 0};
        for (int i = i0 + (int)threadIdx.x; i <= i1; i += blockDim.x) {
            if (!sel(i)) continue;
            R d0, d1, d2;
            disp(i, d0, d1, d2);
            const R m = tc == 2 ? R(S.mass[i]) : R(1);
            acc[0] += d0 * m; acc[1] += d1 * m; acc[2] += d2 * m; acc[3] += m;
        }
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            for (int o = 16; o > 0; o >>= 1) acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], o);
            if (lane == 0) sw[c][warp] = acc[c];
        }
        __syncthreads();
        if (threadIdx.x < 4) {
            R t = 0;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sw[threadIdx.x][w];
            tot[threadIdx.x] = t;
        }
        __syncthreads();
        if (tot[3] > R(0)) {
            const R dr0 = tot[0] / tot[3], dr1 = tot[1] / tot[3], dr2 = tot[2] / tot[3];
            if (threadIdx.x == 0) e = R(0.5) * fk * (dr0 * dr0 + dr1 * dr1 + dr2 * dr2);
            for (int i = i0 + (int)threadIdx.x; i <= i1; i += blockDim.x) {
                if (!sel(i)) continue;
                const R sc = tc == 1 ? R(S.mass[i]) / R(12.010) : R(1);
                p::grad(S, i, fk * dr0 * sc, fk * dr1 * sc, fk * dr2 * sc);
            }
        }
    } else {
        for (int i = i0 + (int)threadIdx.x; i <= i1; i += blockDim.x) {
            if (!sel(i)) continue;
            R d0, d1, d2;
            disp(i, d0, d1, d2);
            if (T.pbc) {
                // the periodically minimal distance (:15561-15565)
                if (sizeof(R) == 8) {
                    d0 = d0 - R(T.box[0] * round(double(d0) * T.ibox[0]));
                    d1 = d1 - R(T.box[1] * round(double(d1) * T.ibox[1]));
                    d2 = d2 - R(T.box[2] * round(double(d2) * T.ibox[2]));
                } else {
                    d0 = d0 - R(T.boxf[0] * rintf(float(d0) * T.iboxf[0]));
                    d1 = d1 - R(T.boxf[1] * rintf(float(d1) * T.iboxf[1]));
                    d2 = d2 - R(T.boxf[2] * rintf(float(d2) * T.iboxf[2]));
                }
            }
            e += R(0.5) * fk * (d0 * d0 + d1 * d1 + d2 * d2);
            p::grad(S, i, fk * d0, fk * d1, fk * d2);
        }
    }
    const int slots[1] = {EA_RST_PROT};
    long long v[1] = {p::fx(e, S.status)};
    block_energies_fx<1>(S.eacc + (size_t)traj * QG_NE, slots, v, red);
}

// The other restraints of p_restrain (src/md.f90:15580-15800): atom position,
// distance and angle restraints (state-dependent: state 0 adds its energy to
// every state's restraint term, state s only to s with the force weighted by
// lambda_s; distances and angles take the minimum image in a box) and the
// sphere's half-harmonic wall restraints (protein restraint energy).  One
// thread per item; a block holds one trajectory's items.
template <typename R>
__device__ void xrst_block(const DevSys &S, int b, Red &red) {
    typedef P<R> p;
    const int k = b * blockDim.x + threadIdx.x;
    const int traj = S.xr_blk_traj[b];
    const TrajInfo &T = S.traj[traj];
    R est[QG_MAXS], ewall = 0;
#pragma unroll
    for (int s = 0; s < QG_MAXS; ++s) est[s] = 0;
    const int kind = k < S.nxr ? S.xr_kind[k] : -1;
    if (kind >= 0) {
        const int i = S.xr_at[3 * k], j = S.xr_at[3 * k + 1], l = S.xr_at[3 * k + 2], st = S.xr_st[k];
        const double *pd = S.xr_p + 6 * k;
        const float *pf = S.xr_pf + 9 * k;
        const R wgt = st ? p::lambda(T, st - 1) : R(1);
        auto mimg = [&](R &c, int a) {
            if (!T.pbc) return;
            if (sizeof(R) == 8) c = c - R(T.box[a] * round(double(c) * T.ibox[a]));
            else c = c - R(T.boxf[a] * rintf(float(c) * T.iboxf[a]));
        };
        R e = 0;
        if (kind == 0) {
            // atom position restraint: x - x0 per axis, force constants per axis
            R d[3];
            if (sizeof(R) == 8) {
                for (int a = 0; a < 3; ++a) d[a] = R(S.x[3 * i + a] - pd[a]);
            } else {
                const float4 h = S.pos[i], lo = S.poslo[i];
                d[0] = R((h.x - pf[0]) + (lo.x - pf[3]));
                d[1] = R((h.y - pf[1]) + (lo.y - pf[4]));
                d[2] = R((h.z - pf[2]) + (lo.z - pf[5]));
            }
            R fk[3];
            for (int a = 0; a < 3; ++a) fk[a] = sizeof(R) == 8 ? R(pd[3 + a]) : R(pf[6 + a]);
            e = R(0.5) * fk[0] * d[0] * d[0] + R(0.5) * fk[1] * d[1] * d[1] + R(0.5) * fk[2] * d[2] * d[2];
            p::grad(S, i, fk[0] * d[0] * wgt, fk[1] * d[1] * wgt, fk[2] * d[2] * wgt);
        } else if (kind == 1) {
            // distance restraint: flat between d1 and d2, harmonic outside
            const V3<R> v = rel<R>(S, i, j);
            R dr[3] = {v.x, v.y, v.z};
            for (int a = 0; a < 3; ++a) mimg(dr[a], a);
            const R d1 = sizeof(R) == 8 ? R(pd[0]) : R(pf[0]), d2 = sizeof(R) == 8 ? R(pd[1]) : R(pf[1]);
            const R fk = sizeof(R) == 8 ? R(pd[2]) : R(pf[2]);
            const R bl = sqrt(dr[0] * dr[0] + dr[1] * dr[1] + dr[2] * dr[2]);
            R db = 0;
            const bool on = bl < d1 || bl > d2;
            if (bl < d1) db = bl - d1;
            else if (bl > d2) db = bl - d2;
            if (on) {
                e = R(0.5) * fk * db * db;
                const R dv = wgt * fk * db / bl;
                p::grad(S, j, dr[0] * dv, dr[1] * dv, dr[2] * dv);
                p::grad(S, i, -dr[0] * dv, -dr[1] * dv, -dr[2] * dv);
            }
        } else if (kind == 2) {
            // angle restraint i-j-k
            const V3<R> v1 = rel<R>(S, j, i), v2 = rel<R>(S, j, l);
            R a1[3] = {v1.x, v1.y, v1.z}, a2[3] = {v2.x, v2.y, v2.z};
            for (int a = 0; a < 3; ++a) { mimg(a1[a], a); mimg(a2[a], a); }
            const R ang0 = sizeof(R) == 8 ? R(pd[0]) : R(pf[0]), fk = sizeof(R) == 8 ? R(pd[1]) : R(pf[1]);
            const R r2ij = a1[0] * a1[0] + a1[1] * a1[1] + a1[2] * a1[2];
            const R r2jk = a2[0] * a2[0] + a2[1] * a2[1] + a2[2] * a2[2];
            const R rij = sqrt(r2ij), rjk = sqrt(r2jk);
            R scp = (a1[0] * a2[0] + a1[1] * a2[1] + a1[2] * a2[2]) / (rij * rjk);
            if (scp > R(1)) scp = R(1);
            if (scp < R(-1)) scp = R(-1);
            const R theta = acos(scp);
            const R db = theta - ang0 * R(4.0 * atan(1.0) / 180.0);
            e = R(0.5) * fk * db * db;
            const R dv = wgt * fk * db;
            R f1 = sin(theta);
            if (fabs(double(f1)) < QREAL_EPS) f1 = R(QREAL_EPS);
            f1 = R(-1) / f1;
            R di[3], dk[3];
            for (int a = 0; a < 3; ++a) {
                di[a] = f1 * (a2[a] / (rij * rjk) - scp * a1[a] / r2ij);
                dk[a] = f1 * (a1[a] / (rij * rjk) - scp * a2[a] / r2jk);
            }
            p::grad(S, i, dv * di[0], dv * di[1], dv * di[2]);
            p::grad(S, l, dv * dk[0], dv * dk[1], dv * dk[2]);
            p::grad(S, j, -dv * (di[0] + dk[0]), -dv * (di[1] + dk[1]), -dv * (di[2] + dk[2]));
        } else {
            // wall restraint on one atom (the float coordinates are relative to xwcent)
            R dr[3];
            if (sizeof(R) == 8) {
                for (int a = 0; a < 3; ++a) dr[a] = R(S.x[3 * i + a] - T.xwcent[a]);
            } else {
                const float4 h = S.pos[i], lo = S.poslo[i];
                dr[0] = R(h.x + lo.x); dr[1] = R(h.y + lo.y); dr[2] = R(h.z + lo.z);
            }
            R dw, fk, aM, dM;
            if (sizeof(R) == 8) { dw = R(pd[0]); fk = R(pd[1]); aM = R(pd[2]); dM = R(pd[3]); }
            else { dw = R(pf[0]); fk = R(pf[1]); aM = R(pf[2]); dM = R(pf[3]); }
            const R bl = sqrt(dr[0] * dr[0] + dr[1] * dr[1] + dr[2] * dr[2]);
            const R db = bl - dw;
            R dv;
            if (db > R(0)) {
                ewall = R(0.5) * fk * db * db - dM;
                dv = fk * db / bl;
            } else {
                const R fexp = exp(aM * db);
                ewall = dM * (fexp * fexp - R(2) * fexp);
                dv = R(-2) * dM * aM * (fexp - fexp * fexp) / bl;
            }
            p::grad(S, i, dv * dr[0], dv * dr[1], dv * dr[2]);
        }
        if (kind <= 2) {
            if (st == 0) {
                for (int s = 0; s < T.nstates; ++s) est[s] = e;
            } else {
                est[st - 1] = e;
            }
        }
    }
    unsigned long long *ea = S.eacc + (size_t)traj * QG_NE;
    {
        const int slots[1] = {EA_RST_PROT};
        long long v[1] = {p::fx(ewall, S.status)};
        block_energies_fx<1>(ea, slots, v, red);
    }
    for (int s0 = 0; s0 < T.nstates; s0 += 4) {
        int slots[4];
        long long v[4];
        for (int q = 0; q < 4; ++q) {
            const int s = min(s0 + q, T.nstates - 1);
            slots[q] = EA_Q0 + EQ_N * s + EQ_RST;
            v[q] = s0 + q < T.nstates ? p::fx(est[s], S.status) : 0;
        }
        block_energies_fx<4>(ea, slots, v, red);
    }
}

// offdiag, src/md.f90:15444-15470: Hij = A exp(-mu r_kl).  Its only consumer is
// the energy record, so it runs on the FP64 (recorded / drop-in) evaluations.
__device__ void offdiag_block(const DevSys &S, int blk, int od0, int nod) {
    const int kk = blk * blockDim.x + threadIdx.x;
    if (kk >= nod) return;
    const int k = od0 + kk;
    const int traj = S.od_traj[k];
    const int a = S.q_atom[S.od_kl[2 * k]], b = S.q_atom[S.od_kl[2 * k + 1]];
    const V3<double> d = rel<double>(S, a, b);
    const double r = sqrt(d.x * d.x + d.y * d.y + d.z * d.z);
    const int slot = S.od_ij[2 * k];   // index of the coupling within its trajectory
    double *o = S.od_out + ((size_t)traj * QG_MAXOD + slot) * 2;
    o[0] = S.od_Amu[2 * k] * exp(-S.od_Amu[2 * k + 1] * r);
    o[1] = r;
}

// The small terms share one launch: consecutive block ranges select the term.
struct MiscPlan {
    int nqq, nbt, nfix, nrad, nqb, nod, nrs, nxr;    // blocks per term
    // the tables' part of the batch (BlockTables ranges): first classical
    // bonded block, Q bonded terms [qt0, qt0 + nqt), off-diagonal items
    // [od0, od0 + nodi), first sequence restraint, first p_restrain block
    int bt0, qt0, nqt, od0, nodi, rs0, xr0;
};

template <typename R>
__device__ __forceinline__ void misc_body(const DevSys &S, const MiscPlan &P, const int *qq_traj, const int *qq_s,
                                          const int *satom, const int *wgrp, Red &red) {
    int b = blockIdx.x;
    if (b < P.nqq) { qq_block<R>(S, b, qq_traj, qq_s, red); return; }
    b -= P.nqq;
    if (b < P.nbt) { bonded_block<R>(S, b + P.bt0, red); return; }
    b -= P.nbt;
    if (b < P.nfix) { fix_shell_block<R>(S, b, satom, red); return; }
    b -= P.nfix;
    if (b < P.nrad) { restrain_solvent_block<R>(S, b, wgrp, red); return; }
    b -= P.nrad;
    if (b < P.nqb) { qbonded_block<R>(S, b, P.qt0, P.nqt); return; }
    b -= P.nqb;
    if (b < P.nrs) { seqrst_block<R>(S, b + P.rs0, red); return; }
    b -= P.nrs;
    if (b < P.nxr) { xrst_block<R>(S, b + P.xr0, red); return; }
    b -= P.nxr;
    if (sizeof(R) == 8 && b < P.nod) offdiag_block(S, b, P.od0, P.nodi);
}

__global__ void __launch_bounds__(QG_BLOCK) k_misc(DevSys S, MiscPlan P, const int *qq_traj, const int *qq_s,
                                                   const int *satom, const int *wgrp, EaccSel esel) {
    __shared__ Red red;
    bool acc = esel.mode == EACC_FP64;
    if (esel.mode == EACC_RECORD) acc = esel.ene_every > 0 && ((esel.recctl[0] + esel.k) % esel.ene_every) == 0;
    if (acc) misc_body<double>(S, P, qq_traj, qq_s, satom, wgrp, red);
    else misc_body<float>(S, P, qq_traj, qq_s, satom, wgrp, red);
}

static inline int nblk(int n, int b) { return (n + b - 1) / b; }

void launch_misc(const DevSys &S, const BlockTables &B, LaunchCtx &L, int terms, EaccSel e) {
    MiscPlan P{};
    P.nqq = (terms & QGPU_TERMS_QQ) ? B.nqqblk : 0;
    P.nbt = (terms & QGPU_TERMS_BONDED) ? B.nbtblk : 0;
    P.nfix = (terms & QGPU_TERMS_RESTRAINT) ? B.nsatom / QG_BLOCK : 0;
    P.nrad = (terms & QGPU_TERMS_RESTRAINT) ? B.nwgrp / QG_BLOCK : 0;
    P.nqb = (terms & QGPU_TERMS_QBONDED) ? nblk(B.nqt * QG_MAXS, QG_BLOCK) : 0;
    P.nod = nblk(B.nod, QG_BLOCK);
    P.nrs = (terms & QGPU_TERMS_RESTRAINT) ? B.nrs : 0;
    P.bt0 = B.bt0; P.qt0 = B.qt0; P.nqt = B.nqt; P.od0 = B.od0; P.nodi = B.nod; P.rs0 = B.rs0; P.xr0 = B.xr0;
    P.nxr = (terms & QGPU_TERMS_RESTRAINT) ? B.nxrblk : 0;
    const int nb = P.nqq + P.nbt + P.nfix + P.nrad + P.nqb + P.nod + P.nrs + P.nxr;
    if (!nb) return;
    prof_begin(L, "k_misc");
    k_misc<<<nb, QG_BLOCK, 0, L.stream>>>(S, P, B.qqblk_traj, B.qqblk_s, B.satom, B.wgrp, e);
    prof_end(L);
    (*L.nlaunch)++;
}

// ------------------------------------------------------------------ watpol
// watpol, src/md.f90:18372-18541: radial polarisation restraint of the waters
// in the outer shells, one block per trajectory with the restraint on, FP64
// throughout.  Coordinates are the origin-relative hi + lo floats (always
// current; the origin is the solvent centre).  The reference's selection
// sort by theta (ties in water order) is a rank: the number of shell members
// with a smaller (theta, water) key.  Per-trajectory scratch (e_th, e_iw,
// e_sh, e_rank, srt) lives in wp_scr at TrajInfo::wp_scr0.
struct WpWater {
    double rmu[3], rcu[3], rm, rc, scp, theta;
};
__device__ __forceinline__ void wp_water(const DevSys &S, int o, WpWater &w) {
    double x[3][3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float4 h = S.pos[o + k], l = S.poslo[o + k];
        x[k][0] = (double)h.x + (double)l.x; x[k][1] = (double)h.y + (double)l.y; x[k][2] = (double)h.z + (double)l.z;
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) { w.rmu[a] = x[1][a] + x[2][a] - 2.0 * x[0][a]; w.rcu[a] = x[0][a]; }
    w.rm = sqrt(w.rmu[0] * w.rmu[0] + w.rmu[1] * w.rmu[1] + w.rmu[2] * w.rmu[2]);
    w.rc = sqrt(w.rcu[0] * w.rcu[0] + w.rcu[1] * w.rcu[1] + w.rcu[2] * w.rcu[2]);
#pragma unroll
    for (int a = 0; a < 3; ++a) { w.rmu[a] /= w.rm; w.rcu[a] /= w.rc; }
    double sc = w.rmu[0] * w.rcu[0] + w.rmu[1] * w.rcu[1] + w.rmu[2] * w.rcu[2];
    sc = fmin(1.0, fmax(-1.0, sc));
    w.scp = sc;
    w.theta = acos(sc);
}

__global__ void __launch_bounds__(QG_WPBLK) k_watpol(DevSys S, const int *wp_traj, double *scr, const int *wp_scr0,
                                                     const int *step_base, int k) {
    __shared__ int cnt[QG_MAXSHELL], tot;
    __shared__ double sred[QG_WPBLK / 32];
    const int tr = wp_traj[blockIdx.x];
    const TrajInfo &T = S.traj[tr];
    const int ns = T.nshell, nw = T.nwat, w0 = T.atom0 + T.nat_solute;
    double *e_th = scr + wp_scr0[blockIdx.x];
    int *e_iw = (int *)(e_th + nw);
    int *e_sh = e_iw + nw;
    int *e_rank = e_sh + nw;
    double *srt = (double *)(e_rank + nw + (nw & 1));
    double *st = S.wp_state + 3 * (size_t)T.wp0;   // per shell: theta_corr, avtheta, avn_insh
    const int tid = threadIdx.x;
    if (tid < QG_MAXSHELL) cnt[tid] = 0;
    if (tid == 0) tot = 0;
    __syncthreads();
    // theta of each water and its shell
    for (int iw = tid; iw < nw; iw += blockDim.x) {
        const int o = w0 + 3 * iw;
        if (S.aexcl[o]) continue;
        WpWater w;
        wp_water(S, o, w);
        if (w.rc > T.wp_rlayer) {
            int is;
            for (is = ns; is >= 2; --is)
                if (w.rc <= T.sh_rout[is - 1]) break;
            if (is < 2) is = 1;
            const int e = atomicAdd(&tot, 1);
            atomicAdd(&cnt[is - 1], 1);
            e_th[e] = w.theta; e_iw[e] = iw; e_sh[e] = is - 1;
        }
    }
    __syncthreads();
    const int ne = tot;
    // rank inside the shell: (theta, water index) order
    for (int e = tid; e < ne; e += blockDim.x) {
        const double t = e_th[e];
        const int iw = e_iw[e], sh = e_sh[e];
        int r = 0;
        for (int f = 0; f < ne; ++f) {
            const double u = e_th[f];
            r += (e_sh[f] == sh) && (u < t || (u == t && e_iw[f] < iw));
        }
        e_rank[e] = r;
        int off = 0;
        for (int q = 0; q < sh; ++q) off += cnt[q];
        srt[off + r] = t;
    }
    // theta_corr update every itdis_update steps (md.f90:18451-18465)
    const int istep = step_base[0] + k;
    if (tid == 0 && istep != 0 && T.itdis_update > 0 && istep % T.itdis_update == 0)
        for (int q = 0; q < ns; ++q) {
            double *sq = st + 3 * q;
            sq[1] /= (double)T.itdis_update;
            sq[2] /= (double)T.itdis_update;
            sq[0] = sq[0] + sq[1] - T.sh_acos_cstb[q];
            sq[1] = 0.0; sq[2] = 0.0;
        }
    __syncthreads();
    // energy and forces
    double esum = 0.0;
    const double pi = 3.141592653589793;
    for (int e = tid; e < ne; e += blockDim.x) {
        const int sh = e_sh[e], n = cnt[sh];
        const int il = e_rank[e] + 1;
        const double arg = 1.0 + (1.0 - 2.0 * (double)il) / (double)n;
        double t0 = acos(arg);
        t0 = t0 - 3.0 * sin(t0) * T.sh_cstb[sh] / 2.0;
        t0 = fmin(pi, fmax(0.0, t0));
        const double dth = e_th[e] - t0 + st[3 * sh];
        esum += 0.5 * T.fkwpol * dth * dth;
        const double dv = T.fkwpol * dth;
        const int o = w0 + 3 * e_iw[e];
        WpWater w;
        wp_water(S, o, w);
        double f0 = sin(acos(w.scp));
        if (fabs(f0) < 1e-14) f0 = 1e-14;
        f0 = dv * (-1.0 / f0);
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const double f1 = (w.rcu[a] - w.rmu[a] * w.scp) / w.rm;
            const double f2 = (w.rmu[a] - w.rcu[a] * w.scp) / w.rc;
            fx_add(S.fx + 3 * o + a, f0 * (-2.0 * f1 + f2), S.status);
            fx_add(S.fx + 3 * (o + 1) + a, f0 * f1, S.status);
            fx_add(S.fx + 3 * (o + 2) + a, f0 * f1, S.status);
        }
    }
    // energy: fixed-point block sum
    long long q = d2fx_chk(esum, S.status);
    for (int o = 16; o > 0; o >>= 1) q += __shfl_xor_sync(0xffffffffu, q, o);
    __shared__ long long qred[QG_WPBLK / 32];
    if ((tid & 31) == 0) qred[tid >> 5] = q;
    __syncthreads();
    if (tid == 0) {
        long long t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += qred[w];
        if (t) atomicAdd(S.eacc + (size_t)tr * QG_NE + EA_RST_WPOL, (unsigned long long)t);
    }
    // shell averages of theta, summed in rank order by one warp per shell
    const int warp = tid >> 5, lane = tid & 31;
    if (warp < ns) {
        int off = 0;
        for (int q2 = 0; q2 < warp; ++q2) off += cnt[q2];
        const int n = cnt[warp];
        double a = 0.0;
        for (int r = lane; r < n; r += 32) a += srt[off + r];
        for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
        if (lane == 0 && n > 0) {
            st[3 * warp + 1] += a / (double)n;
            st[3 * warp + 2] += (double)n;
        }
    }
    (void)sred;
}

void launch_watpol(const DevSys &S, const BlockTables &B, LaunchCtx &L, EaccSel e) {
    if (!B.nwp) return;
    prof_begin(L, "k_watpol");
    k_watpol<<<B.nwp, QG_WPBLK, 0, L.stream>>>(S, B.wp_traj, B.wp_scr, B.wp_scr0, e.recctl, e.k);
    prof_end(L);
    (*L.nlaunch)++;
}
