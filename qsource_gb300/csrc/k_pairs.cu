// k_pairs.cu -- the per-step pair loops of pot_energy_nonbonds
// (src/md.f90:16261-16344), in gather form over the full neighbour lists that
// k_scan builds: every thread owns the atoms of one target and sums all their
// pair terms, so each pair is evaluated from both sides with bitwise opposite
// results and no force atomics are needed inside the loop.  Pair distances come
// from hi/lo float coordinates; energies are Kahan-summed per thread and
// reduced as int64 fixed point; forces go to the int64 fixed-point gradient
// once per atom.  Outside the accurate-energy variants (EACC) these kernels
// execute no FP64 instruction: GB300 issues FP64 at 1/64 of the FP32 rate.
#include "qgpu_internal.cuh"

__device__ __forceinline__ int traj_of_entry(const DevSys &S, int e, bool group) {
    if (e < 0) return -1 - e;
    return group ? S.g_traj[e] : S.atraj[e];
}

__device__ __forceinline__ int ljc(const DevSys &S, const TrajInfo &T, int ta, int tb) {
    return S.ljcod[T.lj0 + (ta - T.type0) * T.natyps + (tb - T.type0)];
}

// lrf_taylor (src/md.f90:5824-5891) for one atom: potential and field of the
// group's Taylor expansion at dr = centre - x.  Adds q*df to the gradient.
__device__ __forceinline__ float lrf_atom(const float *ph, float dx, float dy, float dz, float q, float &gx, float &gy,
                                          float &gz) {
    const float p2x = ph[4] * dx + ph[7] * dy + ph[8] * dz;
    const float p2y = ph[7] * dx + ph[5] * dy + ph[9] * dz;
    const float p2z = ph[8] * dx + ph[9] * dy + ph[6] * dz;
    const float V = ph[0] + ph[1] * dx + ph[2] * dy + ph[3] * dz + 0.5f * (p2x * dx + p2y * dy + p2z * dz);
    const float xx = dx * dx, yy = dy * dy, zz = dz * dz, xy = dx * dy, xz = dx * dz, yz = dy * dz;
    // phi3 order: xxx yyy zzz xxy xxz xyy xzz yyz yzz xyz
    const float tx = ph[10] * xx + ph[15] * yy + ph[16] * zz + 2.f * (ph[13] * xy + ph[14] * xz + ph[19] * yz);
    const float ty = ph[13] * xx + ph[11] * yy + ph[18] * zz + 2.f * (ph[15] * xy + ph[19] * xz + ph[17] * yz);
    const float tz = ph[14] * xx + ph[17] * yy + ph[12] * zz + 2.f * (ph[19] * xy + ph[16] * xz + ph[18] * yz);
    gx -= q * (ph[1] + p2x + 0.5f * tx);
    gy -= q * (ph[2] + p2y + 0.5f * ty);
    gz -= q * (ph[3] + p2z + 0.5f * tz);
    return 0.5f * q * V;
}

// FP64 reciprocal square root and reciprocal by Newton-Raphson iteration
// from an FP32 hardware estimate: y <- y (3 - x y^2) / 2 and y <- y (2 - x y)
// square the relative error each step, so two steps take the FP32 estimate's
// ~1e-7 below FP64 rounding.  The FP64 energy paths use them in place of FP64
// rsqrt and division (GB300 issues FP64 at 1/64 of the FP32 rate).
__device__ __forceinline__ double rsqrt_nr(double x) {
    double y = (double)rsqrtf((float)x);
    y = y * (1.5 - 0.5 * x * y * y);
    return y * (1.5 - 0.5 * x * y * y);
}
__device__ __forceinline__ double rcp_nr(double x) {
    double y = (double)__frcp_rn((float)x);
    y = y * (2.0 - x * y);
    return y * (2.0 - x * y);
}

// FP64 squared distance from the master coordinates (accurate-energy mode),
// of the difference x_b - x_a less the pair's periodic shift s (zero in a sphere)
__device__ __forceinline__ double dist2_d(const double *x, int a, int b, const double3 s) {
    const double dx = (x[3 * b] - x[3 * a]) - s.x, dy = (x[3 * b + 1] - x[3 * a + 1]) - s.y,
                 dz = (x[3 * b + 2] - x[3 * a + 2]) - s.z;
    return dx * dx + dy * dy + dz * dz;
}
__device__ __forceinline__ double rinv_d(const double *x, int a, int b, const double3 s) {
    return rsqrt_nr(dist2_d(x, a, b, s));
}
__device__ __forceinline__ double3 dzero3() { return make_double3(0.0, 0.0, 0.0); }

// Energy accumulator of a pair kernel's mode E: 0 Kahan-summed FP32 partials,
// 1 FP64 terms, 2 none (MD steps whose energies nobody reads).
template <int E>
struct EAcc;
template <>
struct EAcc<2> {
    __device__ __forceinline__ void zero() {}
    __device__ __forceinline__ void term(float, double) {}
    __device__ __forceinline__ void flush() {}
    __device__ __forceinline__ long long fx(float, int *) const { return 0; }
};
template <>
struct EAcc<0> {
    KSum k;
    float part;
    __device__ __forceinline__ void zero() { k.zero(); part = 0.f; }
    __device__ __forceinline__ void term(float f, double) { part += f; }
    __device__ __forceinline__ void flush() { k.add(part); part = 0.f; }
    __device__ __forceinline__ long long fx(float scale, int *st) const { return k.fx(scale, st); }
};
template <>
struct EAcc<1> {
    double s;
    __device__ __forceinline__ void zero() { s = 0.0; }
    __device__ __forceinline__ void term(float, double d) { s += d; }
    __device__ __forceinline__ void flush() {}
    __device__ __forceinline__ long long fx(float scale, int *st) const { return d2fx_chk(s * (double)scale, st); }
};

// --------------------------------------------------------------- waters
// nonbond_ww_spc (src/md.f90:15021-15119), the water side of nonbond_pw
// (13282-13365) and lrf_taylor for the three water atoms.
// LW lanes share one water: lane l takes neighbours l, l+LW, ...; the
// lanes' partial gradients are summed by an xor butterfly (fixed order).
// BOX: some trajectory of the batch is a periodic box (its kernels subtract
// the pair shifts; sphere trajectories of the batch have a zero box).
template <int E, int LW, int MINB, int U, bool BOX>
__global__ void __launch_bounds__(QG_BLOCK, MINB) k_nb_water(DevSys S, const int *wgrp, int lrf) {
    constexpr bool EACC = E == 1;
    __shared__ long long red[5][QG_BLOCK / 32];
    const int idx = (blockIdx.x * blockDim.x + threadIdx.x) / LW;
    const int lane = threadIdx.x & (LW - 1);
    const int w = wgrp[idx];
    const int traj = traj_of_entry(S, w, true);
    const TrajInfo &T = S.traj[traj];
    EAcc<E> eww_el, eww_vdw, epw_el, epw_vdw;
    eww_el.zero(); eww_vdw.zero(); epw_el.zero(); epw_vdw.zero();
    float elrf = 0.f;
    const bool valid = w >= 0 && !S.g_excl[w];
    int a0 = 0;
    float gx[3] = {0, 0, 0}, gy[3] = {0, 0, 0}, gz[3] = {0, 0, 0};
    // the water's own packed record: O hi/lo and the H offsets
    float4 r0 = make_float4(0, 0, 0, 0), r1 = r0, r2 = r0;
    if (valid) {
        a0 = S.g_atoms[S.g_start[w]];
        int ta[3];
        double qd[3] = {0, 0, 0};
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            ta[a] = S.atype[a0 + a];
            if (EACC) qd[a] = S.crg_d[a0 + a];
        }
        const int n = S.nb_count[w], nw = S.nb_nw[w];
        const int *lst = S.nb_list + (size_t)w * S.nb_cap;
        const float wwA = T.ww_A, wwB = T.ww_B;
        // water neighbours: 3x3 SPC pairs with the charge products of the
        // solvent table, LJ on O-O only (nonbond_ww_spc).  Both waters come
        // from their packed records: O as hi/lo, H as float offsets from O.
        // d = dO + (db - da) is formed so that the opposite side of the pair
        // computes exactly -d.
        float qq[9];
#pragma unroll
        for (int c = 0; c < 9; ++c) qq[c] = T.wwqq[c];
        r0 = S.wrec[a0]; r1 = S.wrec[a0 + 1]; r2 = S.wrec[a0 + 2];
        const float3 da[3] = {make_float3(0.f, 0.f, 0.f), make_float3(r0.w, r1.w, r2.x), make_float3(r2.y, r2.z, r2.w)};
        const bool pbc = BOX && T.pbc != 0;
        auto ww = [&](int b0, const float4 q0, const float4 q1, const float4 q2) {
            float3 dO = make_float3((q0.x - r0.x) + (q1.x - r1.x), (q0.y - r0.y) + (q1.y - r1.y),
                                    (q0.z - r0.z) + (q1.z - r1.z));
            // box: the O-O image fixes all nine pairs (nonbond_ww_spc_box :15187-15193)
            double3 shd = dzero3();
            if (pbc) {
                dO = f3sub(dO, box_shift(T, dO));
                if (EACC) shd = box_shift_d(T, S.x, a0, b0);
            }
            const float3 db[3] = {make_float3(0.f, 0.f, 0.f), make_float3(q0.w, q1.w, q2.x),
                                  make_float3(q2.y, q2.z, q2.w)};
#pragma unroll
            for (int a = 0; a < 3; ++a) {
#pragma unroll
                for (int b = 0; b < 3; ++b) {
                    const float3 d = make_float3(dO.x + (db[b].x - da[a].x), dO.y + (db[b].y - da[a].y),
                                                 dO.z + (db[b].z - da[a].z));
                    const float r2 = d.x * d.x + d.y * d.y + d.z * d.z;
                    const float ri = rsqrtf(r2), ri2 = ri * ri;
                    const float Vel = qq[3 * a + b] * ri;
                    float dv = -Vel * ri2;
                    double rid = 0.0;
                    if (EACC) rid = rinv_d(S.x, a0 + a, b0 + b, shd);
                    if (a == 0 && b == 0) {
                        const float r6 = ri2 * ri2 * ri2;
                        const float Va = wwA * r6 * r6, Vb = wwB * r6;
                        dv += ri2 * (-12.f * Va + 6.f * Vb);
                        double ed = 0.0;
                        if (EACC) {
                            const double r6d = rid * rid * rid * rid * rid * rid;
                            ed = T.ww_Ad * r6d * r6d - T.ww_Bd * r6d;
                        }
                        eww_vdw.term(Va - Vb, ed);
                    }
                    eww_el.term(Vel, EACC ? qd[a] * S.crg_d[b0 + b] * rid : 0.0);
                    gx[a] -= dv * d.x; gy[a] -= dv * d.y; gz[a] -= dv * d.z;
                }
            }
            eww_el.flush(); eww_vdw.flush();
        };
        // U neighbours per iteration keep U sets of loads in flight; U == 3 is
        // a software pipeline instead: while one neighbour computes, the next
        // one's record and the index after it are in flight
        int k = lane;
        if (U == 3) {
            if (k < nw) {
                int b = lst[k];
                float4 q0 = S.wrec[b], q1 = S.wrec[b + 1], q2 = S.wrec[b + 2];
                int bn = k + LW < nw ? lst[k + LW] : 0;
                for (;;) {
                    const bool more = k + LW < nw;
                    float4 n0 = make_float4(0.f, 0.f, 0.f, 0.f), n1 = n0, n2 = n0;
                    int bnn = 0;
                    if (more) {
                        n0 = S.wrec[bn]; n1 = S.wrec[bn + 1]; n2 = S.wrec[bn + 2];
                        if (k + 2 * LW < nw) bnn = lst[k + 2 * LW];
                    }
                    ww(b, q0, q1, q2);
                    if (!more) break;
                    k += LW; b = bn; bn = bnn; q0 = n0; q1 = n1; q2 = n2;
                }
            }
            k = nw;
        }
        for (; U != 3 && k + (U - 1) * LW < nw; k += U * LW) {
            int bb[U];
            float4 p[U][3];
#pragma unroll
            for (int u = 0; u < U; ++u) bb[u] = lst[k + u * LW];
#pragma unroll
            for (int u = 0; u < U; ++u) { p[u][0] = S.wrec[bb[u]]; p[u][1] = S.wrec[bb[u] + 1]; p[u][2] = S.wrec[bb[u] + 2]; }
#pragma unroll
            for (int u = 0; u < U; ++u) ww(bb[u], p[u][0], p[u][1], p[u][2]);
        }
        for (; k < nw; k += LW) {
            const int b0 = lst[k];
            ww(b0, S.wrec[b0], S.wrec[b0 + 1], S.wrec[b0 + 2]);
        }
        // solute neighbours (the water side of nonbond_pw).  d = dpos(O, j) - d_a
        // is the exact negative of the solute side's dpos(j, O) + d_a.
        const float4 oh = make_float4(r0.x, r0.y, r0.z, 0.f), ol = make_float4(r1.x, r1.y, r1.z, 0.f);
        for (int kk = nw + lane; kk < n; kk += LW) {
            const int g = lst[kk];
            // box: the image of the group's switch atom relative to this O
            // (nonbond_pw_box :13395-13405); with any-atom lists the solute
            // atom of the pair's shift record (nbpwlis2_box_lrf :8835-8836)
            float3 sg = make_float3(0.f, 0.f, 0.f);
            double3 sgd = dzero3();
            if (pbc) {
                const int sw = T.any_atom ? S.nb_sha[(size_t)w * S.nb_cap + kk].y : S.g_switch[g];
                sg = box_shift(T, dpos(oh, ol, S.pos[sw], S.poslo[sw]));
                if (EACC) sgd = box_shift_d(T, S.x, a0, sw);
            }
            for (int q = S.g_start[g]; q < S.g_start[g + 1]; ++q) {
                const int b = S.g_atoms[q];
                if (S.aq[b] >= 0) continue;
                const float4 bh = S.pos[b], bl = S.poslo[b];
                const int tb = S.atype[b];
                const float3 dO = f3sub(dpos(oh, ol, bh, bl), sg);
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    const int c = ljc(S, T, ta[a], tb);
                    const int li = lj_index(T, ta[a], tb, c);
                    const float A = S.ljA[li], B = S.ljB[li];
                    const float3 d = make_float3(dO.x - da[a].x, dO.y - da[a].y, dO.z - da[a].z);
                    const float r2 = d.x * d.x + d.y * d.y + d.z * d.z;
                    const float ri = rsqrtf(r2), ri2 = ri * ri, r6 = ri2 * ri2 * ri2;
                    const float Vel = T.chg_solv[a] * bh.w * ri, Va = A * r6 * r6, Vb = B * r6;
                    const float dv = ri2 * (-Vel - 12.f * Va + 6.f * Vb);
                    double eld = 0.0, evd = 0.0;
                    if (EACC) {
                        const double rid = rinv_d(S.x, a0 + a, b, sgd), r6d = rid * rid * rid * rid * rid * rid;
                        eld = qd[a] * S.crg_d[b] * rid;
                        evd = S.ljA_d[li] * r6d * r6d - S.ljB_d[li] * r6d;
                    }
                    epw_el.term(Vel, eld); epw_vdw.term(Va - Vb, evd);
                    gx[a] -= dv * d.x; gy[a] -= dv * d.y; gz[a] -= dv * d.z;
                }
            }
            epw_el.flush(); epw_vdw.flush();
        }
    }
    // every lane of the warp takes part in the butterfly (invalid lanes add 0)
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int o = LW / 2; o > 0; o >>= 1) {
            gx[a] += __shfl_xor_sync(S_GROUP_MASK, gx[a], o, LW);
            gy[a] += __shfl_xor_sync(S_GROUP_MASK, gy[a], o, LW);
            gz[a] += __shfl_xor_sync(S_GROUP_MASK, gz[a], o, LW);
        }
    // after the butterfly every lane holds the three sums: lane a (0..2)
    // adds the Taylor term of atom a and stores its gradient
    if (valid && lane < 3) {
        const int a = lane;
        float fx = a == 0 ? gx[0] : (a == 1 ? gx[1] : gx[2]);
        float fy = a == 0 ? gy[0] : (a == 1 ? gy[1] : gy[2]);
        float fz = a == 0 ? gz[0] : (a == 1 ? gz[1] : gz[2]);
        if (lrf) {
            const float *ph = S.g_phif + (size_t)w * QG_NPHI;
            const float4 c = S.g_centf[w];
            // centre - x_a = ((c - O_hi) - O_lo) - d_a
            const float3 da = a == 0 ? make_float3(0.f, 0.f, 0.f)
                                     : (a == 1 ? make_float3(r0.w, r1.w, r2.x) : make_float3(r2.y, r2.z, r2.w));
            elrf += lrf_atom(ph, ((c.x - r0.x) - r1.x) - da.x, ((c.y - r0.y) - r1.y) - da.y,
                             ((c.z - r0.z) - r1.z) - da.z, T.chg_solv[a], fx, fy, fz);
        }
        fx_addf(S.fx + 3 * (a0 + a), fx, S.status);
        fx_addf(S.fx + 3 * (a0 + a) + 1, fy, S.status);
        fx_addf(S.fx + 3 * (a0 + a) + 2, fz, S.status);
    }
    if (E == 2) return;   // no energies on this step
    // pair energies are summed from both sides: half of each thread's sum
    const int slots[5] = {EA_WW_EL, EA_WW_VDW, EA_PW_EL, EA_PW_VDW, EA_LRF};
    long long ev[5] = {eww_el.fx(0.5f, S.status), eww_vdw.fx(0.5f, S.status), epw_el.fx(0.5f, S.status),
                       epw_vdw.fx(0.5f, S.status), f2fx_chk(elrf, S.status)};
    block_energies_fx<5>(S.eacc + (size_t)traj * QG_NE, slots, ev, red);
}

// Water-water LJ of the eight atom pairs beside O-O, for trajectories whose
// water hydrogens carry LJ under the arithmetic rule (nonbon2_ww,
// src/md.f90:12847-12944, takes LJ on all nine pairs; k_nb_water has the
// Coulomb terms of all nine and the O-O LJ).  LW lanes per water over its
// water neighbours, the same relative vectors and periodic image as
// k_nb_water; the forces of this water's atoms, and half of each pair energy
// (the pair is met from both sides).
template <int E, bool BOX>
__global__ void __launch_bounds__(QG_BLOCK) k_ww_hlj(DevSys S, const int *wgrp) {
    constexpr int LW = 8;
    constexpr bool EACC = E == 1;
    __shared__ long long red[1][QG_BLOCK / 32];
    const int idx = (blockIdx.x * blockDim.x + threadIdx.x) / LW;
    const int lane = threadIdx.x & (LW - 1);
    const int w = wgrp[idx];
    const int traj = traj_of_entry(S, w, true);
    const TrajInfo &T = S.traj[traj];
    EAcc<E> evdw;
    evdw.zero();
    const bool valid = w >= 0 && !S.g_excl[w] && T.hlj;
    int a0 = 0;
    float gx[3] = {0, 0, 0}, gy[3] = {0, 0, 0}, gz[3] = {0, 0, 0};
    if (valid) {
        a0 = S.g_atoms[S.g_start[w]];
        const int nw = S.nb_nw[w];
        const int *lst = S.nb_list + (size_t)w * S.nb_cap;
        const float4 r0 = S.wrec[a0], r1 = S.wrec[a0 + 1], r2 = S.wrec[a0 + 2];
        const float3 da[3] = {make_float3(0.f, 0.f, 0.f), make_float3(r0.w, r1.w, r2.x), make_float3(r2.y, r2.z, r2.w)};
        const bool pbc = BOX && T.pbc != 0;
        for (int k = lane; k < nw; k += LW) {
            const int b0 = lst[k];
            const float4 q0 = S.wrec[b0], q1 = S.wrec[b0 + 1], q2 = S.wrec[b0 + 2];
            float3 dO = make_float3((q0.x - r0.x) + (q1.x - r1.x), (q0.y - r0.y) + (q1.y - r1.y),
                                    (q0.z - r0.z) + (q1.z - r1.z));
            double3 shd = dzero3();
            if (pbc) {
                dO = f3sub(dO, box_shift(T, dO));
                if (EACC) shd = box_shift_d(T, S.x, a0, b0);
            }
            const float3 db[3] = {make_float3(0.f, 0.f, 0.f), make_float3(q0.w, q1.w, q2.x),
                                  make_float3(q2.y, q2.z, q2.w)};
#pragma unroll
            for (int a = 0; a < 3; ++a)
#pragma unroll
                for (int b = 0; b < 3; ++b) {
                    if (a == 0 && b == 0) continue;
                    const float3 d = make_float3(dO.x + (db[b].x - da[a].x), dO.y + (db[b].y - da[a].y),
                                                 dO.z + (db[b].z - da[a].z));
                    const float r2f = d.x * d.x + d.y * d.y + d.z * d.z;
                    const float ri = rsqrtf(r2f), ri2 = ri * ri, r6 = ri2 * ri2 * ri2;
                    const float Va = T.wwh_A[3 * a + b] * r6 * r6, Vb = T.wwh_B[3 * a + b] * r6;
                    const float dv = ri2 * (-12.f * Va + 6.f * Vb);
                    double ed = 0.0;
                    if (EACC) {
                        const double rid = rinv_d(S.x, a0 + a, b0 + b, shd);
                        const double r6d = rid * rid * rid * rid * rid * rid;
                        ed = T.wwh_Ad[3 * a + b] * r6d * r6d - T.wwh_Bd[3 * a + b] * r6d;
                    }
                    evdw.term(Va - Vb, ed);
                    gx[a] -= dv * d.x; gy[a] -= dv * d.y; gz[a] -= dv * d.z;
                }
            evdw.flush();
        }
    }
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int o = LW / 2; o > 0; o >>= 1) {
            gx[a] += __shfl_xor_sync(0xffffffffu, gx[a], o, LW);
            gy[a] += __shfl_xor_sync(0xffffffffu, gy[a], o, LW);
            gz[a] += __shfl_xor_sync(0xffffffffu, gz[a], o, LW);
        }
    if (valid && lane < 3) {
        const int a = lane;
        const float fx = a == 0 ? gx[0] : (a == 1 ? gx[1] : gx[2]);
        const float fy = a == 0 ? gy[0] : (a == 1 ? gy[1] : gy[2]);
        const float fz = a == 0 ? gz[0] : (a == 1 ? gz[1] : gz[2]);
        fx_addf(S.fx + 3 * (a0 + a), fx, S.status);
        fx_addf(S.fx + 3 * (a0 + a) + 1, fy, S.status);
        fx_addf(S.fx + 3 * (a0 + a) + 2, fz, S.status);
    }
    if (E == 2) return;
    const int slots[1] = {EA_WW_VDW};
    long long ev[1] = {evdw.fx(0.5f, S.status)};
    block_energies_fx<1>(S.eacc + (size_t)traj * QG_NE, slots, ev, red);
}

// ------------------------------------------------------- solute atoms
struct PairFlags { bool excl, p14; };

__device__ __forceinline__ PairFlags pair_flags(const DevSys &S, int i, int j) {
    PairFlags f{false, false};
    const int rel = j - i;
    if (rel >= -32 && rel < 32) {
        f.excl = (S.exmask[i] >> (rel + 32)) & 1ull;
        f.p14 = (S.p14mask[i] >> (rel + 32)) & 1ull;
    } else {
        for (int k = S.exlong_first[i]; k < S.exlong_first[i + 1]; ++k)
            if (S.exlong_j[k] == j) {
                if (S.exlong_kind[k]) f.p14 = true; else f.excl = true;
            }
    }
    return f;
}

// nonbond_pp (src/md.f90:13069-13155) and the solute side of nonbond_pw, plus
// lrf_taylor, for one non-Q solute atom.  Per pair: LJ code c (3 = a 1-4 pair
// with the el14 factor, nonbond_pp :13102-13111) and the periodic shift (sf,
// sd) of the group pair (nonbond_pp_box :13226-13228).
#ifndef QG_PPB
#define QG_PPB 4   // solute atoms of a neighbour group loaded together
#endif
#ifndef QG_SOL_MINB
#define QG_SOL_MINB 1   // k_nb_solute register bound (minimum resident blocks)
#endif
template <int E, int LW, bool BOX>
__global__ void __launch_bounds__(QG_BLOCK, QG_SOL_MINB) k_nb_solute(DevSys S, const int *satom, int lrf) {
    constexpr bool EACC = E == 1;
    __shared__ long long red[5][QG_BLOCK / 32];
    const int idx = (blockIdx.x * blockDim.x + threadIdx.x) / LW;
    const int lane = threadIdx.x & (LW - 1);
    const int i = satom[idx];
    const int traj = traj_of_entry(S, i, false);
    const TrajInfo &T = S.traj[traj];
    EAcc<E> epp_el, epp_vdw, epw_el, epw_vdw;
    epp_el.zero(); epp_vdw.zero(); epw_el.zero(); epw_vdw.zero();
    float elrf = 0.f;
    const bool valid = i >= 0 && S.aq[i] < 0 && !S.g_excl[S.agrp[i]];
    float gx = 0.f, gy = 0.f, gz = 0.f;
    int g = 0;
    float4 ih = {}, il = {};
    if (valid) {
        g = S.agrp[i];
        ih = S.pos[i]; il = S.poslo[i];
        const int ti = S.atype[i];
        const double qi = EACC ? S.crg_d[i] : 0.0;
        const float el14 = T.el14;
        const bool pbc = BOX && T.pbc != 0;
        const int swg = S.g_switch[g];
        float4 swh = {}, swl = {};
        if (pbc) { swh = S.pos[swg]; swl = S.poslo[swg]; }
        // pp pairs with exclusion / 1-4 handling (nbpplist_lrf :8108-8166):
        // the atoms of a neighbour group in batches of QG_PPB, each batch's
        // records, types, LJ codes and LJ products loaded together before any
        // pair is formed (the loads of a batch are in flight at once)
        const unsigned long long exm = S.exmask[i], p14m = S.p14mask[i];
        const int ljrow = T.lj0 + (ti - T.type0) * T.natyps - T.type0;
        auto pp_range = [&](int a0, int a1, int step, const float3 sf, const double3 sd) {
            for (int kk = a0; kk < a1; kk += QG_PPB * step) {
                int jj[QG_PPB], cc[QG_PPB];
                float4 jh[QG_PPB], jl[QG_PPB];
                float2 ab[QG_PPB];
#pragma unroll
                for (int u = 0; u < QG_PPB; ++u) jj[u] = kk + u * step < a1 ? S.g_atoms[kk + u * step] : -1;
#pragma unroll
                for (int u = 0; u < QG_PPB; ++u) {
                    cc[u] = -1;   // else (type << 2) | LJ code (1, 2; 3 = 1-4 pair)
                    if (jj[u] < 0 || jj[u] == i || S.aq[jj[u]] >= 0) continue;
                    const int j = jj[u], rel = j - i;
                    bool excl, p14;
                    if (rel >= -32 && rel < 32) {
                        excl = (exm >> (rel + 32)) & 1ull;
                        p14 = (p14m >> (rel + 32)) & 1ull;
                    } else {
                        const PairFlags f = pair_flags(S, i, j);
                        excl = f.excl; p14 = f.p14;
                    }
                    if (excl) continue;
                    jh[u] = S.pos[j]; jl[u] = S.poslo[j];
                    const int tj = S.atype[j];
                    cc[u] = (tj << 2) | (p14 ? 3 : S.ljcod[ljrow + tj]);
                }
#pragma unroll
                for (int u = 0; u < QG_PPB; ++u)
                    if (cc[u] >= 0) {
                        const int li = (ljrow + (cc[u] >> 2)) * 3 + (cc[u] & 3) - 1;
                        ab[u] = make_float2(S.ljA[li], S.ljB[li]);
                    }
#pragma unroll
                for (int u = 0; u < QG_PPB; ++u) {
                    if (cc[u] < 0) continue;
                    const int j = jj[u], c = cc[u] & 3;
                    const float3 d = f3sub(dpos(ih, il, jh[u], jl[u]), sf);
                    const float r2 = d.x * d.x + d.y * d.y + d.z * d.z;
                    const float ri = rsqrtf(r2), ri2 = ri * ri, r6 = ri2 * ri2 * ri2;
                    float Vel = ih.w * jh[u].w * ri;
                    if (c == 3) Vel *= el14;
                    const float Va = ab[u].x * r6 * r6, Vb = ab[u].y * r6;
                    const float dv = ri2 * (-Vel - 12.f * Va + 6.f * Vb);
                    double eld = 0.0, evd = 0.0;
                    if (EACC) {
                        const int li = (ljrow + (cc[u] >> 2)) * 3 + c - 1;
                        const double rid = rinv_d(S.x, i, j, sd), r6d = rid * rid * rid * rid * rid * rid;
                        eld = qi * S.crg_d[j] * rid;
                        if (c == 3) eld *= (double)T.el14d;
                        evd = S.ljA_d[li] * r6d * r6d - S.ljB_d[li] * r6d;
                    }
                    epp_el.term(Vel, eld); epp_vdw.term(Va - Vb, evd);
                    gx -= dv * d.x; gy -= dv * d.y; gz -= dv * d.z;
                }
            }
        };
        const float3 zf = make_float3(0.f, 0.f, 0.f);
        pp_range(S.g_start[g] + lane, S.g_start[g + 1], LW, zf, dzero3());
        epp_el.flush(); epp_vdw.flush();
        const int n = S.nb_count[g], nw = S.nb_nw[g];
        const int *lst = S.nb_list + (size_t)g * S.nb_cap;
        // water neighbours from their packed records: d = dpos(i, O) + d_k;
        // LJ products and charge products of the three water atoms formed once
        // (all waters of a trajectory share types and charges)
        float Aw[3], Bw[3], qw[3];
        int cw[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const int tw = S.atype[T.atom0 + T.nat_solute + k];
            cw[k] = ljc(S, T, ti, tw);
            Aw[k] = S.ljA[lj_index(T, ti, tw, cw[k])];
            Bw[k] = S.ljB[lj_index(T, ti, tw, cw[k])];
            qw[k] = ih.w * T.chg_solv[k];
        }
        for (int k = lane; k < nw; k += LW) {
            const int b0 = lst[k];
            const float4 w0 = S.wrec[b0], w1 = S.wrec[b0 + 1], w2 = S.wrec[b0 + 2];
            const float4 oh = make_float4(w0.x, w0.y, w0.z, 0.f), ol = make_float4(w1.x, w1.y, w1.z, 0.f);
            float3 dO = dpos(ih, il, oh, ol);
            // box: the O image relative to this group's switch atom (nonbond_pw_box);
            // with any-atom lists relative to the solute atom of the pair's
            // shift record (nbpwlis2_box_lrf :8835-8836)
            double3 sgd = dzero3();
            if (pbc) {
                if (T.any_atom) {
                    const int sa = S.nb_sha[(size_t)g * S.nb_cap + k].x;
                    dO = f3sub(dO, box_shift(T, dpos(S.pos[sa], S.poslo[sa], oh, ol)));
                    if (EACC) sgd = box_shift_d(T, S.x, sa, b0);
                } else {
                    dO = f3sub(dO, box_shift(T, dpos(swh, swl, oh, ol)));
                    if (EACC) sgd = box_shift_d(T, S.x, swg, b0);
                }
            }
            const float3 dk[3] = {make_float3(0.f, 0.f, 0.f), make_float3(w0.w, w1.w, w2.x), make_float3(w2.y, w2.z, w2.w)};
#pragma unroll
            for (int b = 0; b < 3; ++b) {
                const float3 d = make_float3(dO.x + dk[b].x, dO.y + dk[b].y, dO.z + dk[b].z);
                const float r2 = d.x * d.x + d.y * d.y + d.z * d.z;
                const float ri = rsqrtf(r2), ri2 = ri * ri, r6 = ri2 * ri2 * ri2;
                const float Vel = qw[b] * ri, Va = Aw[b] * r6 * r6, Vb = Bw[b] * r6;
                const float dv = ri2 * (-Vel - 12.f * Va + 6.f * Vb);
                double eld = 0.0, evd = 0.0;
                if (EACC) {
                    const int j = b0 + b, tj = S.atype[j];
                    const double rid = rinv_d(S.x, i, j, sgd), r6d = rid * rid * rid * rid * rid * rid;
                    eld = qi * S.crg_d[j] * rid;
                    const int li = lj_index(T, ti, tj, cw[b]);
                    evd = S.ljA_d[li] * r6d * r6d - S.ljB_d[li] * r6d;
                }
                epw_el.term(Vel, eld); epw_vdw.term(Va - Vb, evd);
                gx -= dv * d.x; gy -= dv * d.y; gz -= dv * d.z;
            }
            epw_el.flush(); epw_vdw.flush();
        }
        for (int k = nw + lane; k < n; k += LW) {
            const int h = lst[k];
            float3 sf = zf;
            double3 sd = dzero3();
            if (pbc) {
                // the switch atoms of the group pair; with any-atom lists the
                // pair's shift record (nbpplis2_box_lrf :7338-7339)
                int sa = swg, sb = S.g_switch[h];
                if (T.any_atom) {
                    const int2 r = S.nb_sha[(size_t)g * S.nb_cap + k];
                    sa = r.x; sb = r.y;
                }
                sf = box_shift(T, dpos(S.pos[sa], S.poslo[sa], S.pos[sb], S.poslo[sb]));
                if (EACC) sd = box_shift_d(T, S.x, sa, sb);
            }
            pp_range(S.g_start[h], S.g_start[h + 1], 1, sf, sd);
            epp_el.flush(); epp_vdw.flush();
        }
    }
#pragma unroll
    for (int o = LW / 2; o > 0; o >>= 1) {
        gx += __shfl_xor_sync(S_GROUP_MASK, gx, o, LW);
        gy += __shfl_xor_sync(S_GROUP_MASK, gy, o, LW);
        gz += __shfl_xor_sync(S_GROUP_MASK, gz, o, LW);
    }
    {
        if (valid && lane == 0) {
            if (lrf) {
                const float *ph = S.g_phif + (size_t)g * QG_NPHI;
                const float4 c = S.g_centf[g];
                elrf = lrf_atom(ph, (c.x - ih.x) - il.x, (c.y - ih.y) - il.y, (c.z - ih.z) - il.z, ih.w, gx, gy, gz);
            }
            fx_addf(S.fx + 3 * i, gx, S.status);
            fx_addf(S.fx + 3 * i + 1, gy, S.status);
            fx_addf(S.fx + 3 * i + 2, gz, S.status);
        }
    }
    if (E == 2) return;   // no energies on this step
    const int slots[5] = {EA_PP_EL, EA_PP_VDW, EA_PW_EL, EA_PW_VDW, EA_LRF};
    long long ev[5] = {epp_el.fx(0.5f, S.status), epp_vdw.fx(0.5f, S.status), epw_el.fx(0.5f, S.status),
                       epw_vdw.fx(0.5f, S.status), f2fx_chk(elrf, S.status)};
    block_energies_fx<5>(S.eacc + (size_t)traj * QG_NE, slots, ev, red);
}

// ------------------------------------------------------- Q-atom loops
// LG lanes share one water (k_qw) or one solute atom (k_qp); lane l takes the
// Q atoms l, l+LG, ...  In each round the lanes of a warp with the same l hold
// partial forces on the same Q atom: an xor butterfly over the groups sums
// them in a fixed order, the warp's sums go to shared memory and the block
// adds its warps in order -- deterministic without float atomics.  LG is
// chosen per launch: more lanes when the Q atoms are many or the items few.
struct QShared {
    float4 qh[QG_MAXQ], ql[QG_MAXQ];
    int qa[QG_MAXQ], qt[QG_MAXQ];   // Q atom index and its LJ type
    float qf[QG_BLOCK / 32][QG_MAXQ][3];
    long long red[2 * QG_MAXS][QG_BLOCK / 32];
};

// sum over the warp's groups of the force on Q atom iq (all lanes call it)
template <int LG>
__device__ __forceinline__ void q_reduce_store(QShared &sh, int iq, bool on, float fx, float fy, float fz) {
#pragma unroll
    for (int o = LG; o < 32; o <<= 1) {
        fx += __shfl_xor_sync(0xffffffffu, fx, o);
        fy += __shfl_xor_sync(0xffffffffu, fy, o);
        fz += __shfl_xor_sync(0xffffffffu, fz, o);
    }
    if ((threadIdx.x & 31) < LG && on) {
        const int w = threadIdx.x >> 5;
        sh.qf[w][iq][0] = fx; sh.qf[w][iq][1] = fy; sh.qf[w][iq][2] = fz;
    }
}
__device__ __forceinline__ void q_flush(const DevSys &S, const TrajInfo &T, QShared &sh) {
    __syncthreads();
    for (int k = threadIdx.x; k < T.nqat * 3; k += blockDim.x) {
        const int iq = k / 3, c = k % 3;
        float s = 0.f;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += sh.qf[w][iq][c];
        if (s != 0.f) fx_addf(S.fx + 3 * S.q_atom[T.q0 + iq] + c, s, S.status);
    }
}
__device__ __forceinline__ void q_load(const DevSys &S, const TrajInfo &T, QShared &sh) {
    for (int k = threadIdx.x; k < T.nqat; k += blockDim.x) {
        const int a = S.q_atom[T.q0 + k];
        sh.qh[k] = S.pos[a]; sh.ql[k] = S.poslo[a];
        sh.qa[k] = a; sh.qt[k] = S.atype[a];
    }
    __syncthreads();
}
// sum of a lane group's partial forces on its own atom
template <int LG>
__device__ __forceinline__ float group_sum(float v) {
#pragma unroll
    for (int o = LG / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ bool eacc_on(const EaccSel &e) {
    if (e.mode == EACC_FP64) return true;
    if (e.mode == EACC_RECORD) return e.ene_every > 0 && ((e.recctl[0] + e.k) % e.ene_every) == 0;
    return false;
}
// energies wanted at all: every drop-in call, and the recorded MD steps
__device__ __forceinline__ bool energies_on(const EaccSel &e) { return e.mode != EACC_RECORD || eacc_on(e); }

// per-state energy sums of one thread: Kahan FP32, or FP64 terms
struct QE {
    KSum k[QG_MAXS];
    double d[QG_MAXS];
    __device__ __forceinline__ void zero() {
#pragma unroll
        for (int s = 0; s < QG_MAXS; ++s) { k[s].zero(); d[s] = 0.0; }
    }
    __device__ __forceinline__ long long fx(int s, bool acc, int *st) const {
        return acc ? d2fx_chk(d[s], st) : k[s].fx(1.f, st);
    }
};

// the per-state el/vdW sums of a Q loop into slots base_el / base_vdw
__device__ __forceinline__ void q_energies(const DevSys &S, int traj, int NS, const QE &eel, const QE &evdw, bool acc,
                                           int e_el, int e_vdw, QShared &sh) {
    int slots[2 * QG_MAXS];
    long long v[2 * QG_MAXS];
#pragma unroll
    for (int s = 0; s < QG_MAXS; ++s) {
        const bool on = s < NS;
        slots[2 * s] = EA_Q0 + EQ_N * s + e_el;
        slots[2 * s + 1] = EA_Q0 + EQ_N * s + e_vdw;
        v[2 * s] = on ? eel.fx(s, acc, S.status) : 0;
        v[2 * s + 1] = on ? evdw.fx(s, acc, S.status) : 0;
    }
    block_energies_fx<2 * QG_MAXS>(S.eacc + (size_t)traj * QG_NE, slots, v, sh.red);
}

// nonbond_qw_spc, src/md.f90:14411-14570.  LG lanes per water.
// E: 0 energies as esel asks (FP32 Kahan or FP64 terms); 2 none (MD steps
// whose energies are not recorded: fewer registers, more resident blocks).
// The per-state O-side constants of every Q atom (A, B, charge, soft-core
// term) are staged in shared memory with the Q positions.
template <int LG, int E, bool HLJ>
__global__ void __launch_bounds__(QG_BLOCK, E == 2 ? 6 : 1) k_qw(DevSys S, const int *wgrp, EaccSel esel) {
    __shared__ QShared sh;
    __shared__ float4 qwp[QG_MAXQ * QG_MAXS];
    const int idx = (blockIdx.x * blockDim.x + threadIdx.x) / LG;
    const int lane = threadIdx.x & (LG - 1);
    const int w = wgrp[idx];
    const int traj = traj_of_entry(S, w, true);
    const TrajInfo &T = S.traj[traj];
    const bool acc = E != 2 && eacc_on(esel), want = E != 2 && energies_on(esel);
    const int ntq = T.natyps + T.nqat;
    for (int k = threadIdx.x; k < T.nqat * QG_MAXS; k += blockDim.x) {
        const int q = T.q0 + k / QG_MAXS, s = k % QG_MAXS;
        const size_t sci = (size_t)T.sc0 + ((size_t)(k / QG_MAXS) * ntq + (size_t)S.qw_sc[q]) * QG_MAXS + s;
        qwp[k] = make_float4(S.qw_A[q * QG_MAXS + s], S.qw_B[q * QG_MAXS + s], S.qcrg_f[q * QG_MAXS + s],
                             T.qvdw ? S.sc_f[sci] : 0.f);
    }
    q_load(S, T, sh);
    const int NS = T.nstates;
    QE eel, evdw;
    eel.zero(); evdw.zero();
    int a0 = -1;
    bool valid = false;
    if (w >= 0) {
        a0 = S.g_atoms[S.g_start[w]];
        valid = S.qw_member[a0] != 0;
    }
    float4 ah[3] = {}, al[3] = {};
    if (valid)
#pragma unroll
        for (int a = 0; a < 3; ++a) { ah[a] = S.pos[a0 + a]; al[a] = S.poslo[a0 + a]; }
    // box: the O image relative to the Q switching atom (nonbond_qw_spc_box :14612-14618)
    float3 sw = make_float3(0.f, 0.f, 0.f);
    double3 swd = dzero3();
    if (valid && T.pbc) {
        sw = box_shift(T, dpos(S.pos[T.qswitch], S.poslo[T.qswitch], ah[0], al[0]));
        if (acc) swd = box_shift_d(T, S.x, T.qswitch, a0);
    }
    float gx[3] = {0, 0, 0}, gy[3] = {0, 0, 0}, gz[3] = {0, 0, 0};
    float lam[QG_MAXS];
#pragma unroll
    for (int s = 0; s < QG_MAXS; ++s) lam[s] = T.lambdaf[s];
    for (int iq0 = 0; iq0 < T.nqat; iq0 += LG) {
        const int iq = iq0 + lane;
        const bool on = iq < T.nqat;
        float qfx = 0.f, qfy = 0.f, qfz = 0.f;
        if (valid && on) {
            const int q = T.q0 + iq;
            const int qa = S.q_atom[q];
            // O: Coulomb + LJ (softcore column = LJ code of the pair, src/md.f90:14492)
            {
                const float3 d = f3sub(dpos(sh.qh[iq], sh.ql[iq], ah[0], al[0]), sw);
                const float r2 = d.x * d.x + d.y * d.y + d.z * d.z;
                const float r6hc = r2 * r2 * r2, ri = rsqrtf(r2), ri2 = ri * ri;
                double rid = 0.0, r6hcd = 0.0;
                if (acc) { const double r2d = dist2_d(S.x, qa, a0, swd); rid = rsqrt_nr(r2d); r6hcd = r2d * r2d * r2d; }
                float dv = 0.f;
#pragma unroll
                for (int s = 0; s < QG_MAXS; ++s) {
                    if (s >= NS) break;
                    const float4 p = qwp[iq * QG_MAXS + s];
                    const float r6s = T.qvdw ? r6hc + p.w : r6hc;
                    const float ir6 = __frcp_rn(r6s);
                    const float Va = p.x * ir6 * ir6, Vb = p.y * ir6;
                    const float Vel = ah[0].w * p.z * ri;
                    dv += lam[s] * ri2 * (-Vel - (12.f * Va - 6.f * Vb) * (r6hc * ir6));
                    if (acc) {
                        const size_t sci = (size_t)T.sc0 + ((size_t)iq * ntq + (size_t)S.qw_sc[q]) * QG_MAXS + s;
                        const double r6sd = T.qvdw ? r6hcd + S.sc_d[sci] : r6hcd;
                        eel.d[s] += S.crg_d[a0] * S.qcrg_d[q * QG_MAXS + s] * rid;
                        const double ir6d = rcp_nr(r6sd);
                        evdw.d[s] += S.qw_Ad[q * QG_MAXS + s] * ir6d * ir6d - S.qw_Bd[q * QG_MAXS + s] * ir6d;
                    } else if (want) {
                        eel.k[s].add(Vel); evdw.k[s].add(Va - Vb);
                    }
                }
                gx[0] += dv * d.x; gy[0] += dv * d.y; gz[0] += dv * d.z;
                qfx -= dv * d.x; qfy -= dv * d.y; qfz -= dv * d.z;
            }
#pragma unroll
            for (int a = 1; a < 3; ++a) {
                const float3 d = f3sub(dpos(sh.qh[iq], sh.ql[iq], ah[a], al[a]), sw);
                const float r2 = d.x * d.x + d.y * d.y + d.z * d.z;
                const float ri = rsqrtf(r2), ri2 = ri * ri;
                const double rid = acc ? rinv_d(S.x, qa, a0 + a, swd) : 0.0;
                float dv = 0.f;
#pragma unroll
                for (int s = 0; s < QG_MAXS; ++s) {
                    if (s >= NS) break;
                    const float Vel = ah[a].w * qwp[iq * QG_MAXS + s].z * ri;
                    if (acc) eel.d[s] += S.crg_d[a0 + a] * S.qcrg_d[q * QG_MAXS + s] * rid;
                    else if (want) eel.k[s].add(Vel);
                    dv -= lam[s] * ri2 * Vel;
                }
                if (HLJ && T.hlj) {
                    // nonbon2_qw (src/md.f90:12562-12695) with LJ on the H:
                    // its products with the Q atom's (state) type, soft-core
                    // column the H's type
                    const float r6hc = r2 * r2 * r2;
                    double r6hcd = 0.0;
                    if (acc) { const double r2d = dist2_d(S.x, qa, a0 + a, swd); r6hcd = r2d * r2d * r2d; }
#pragma unroll
                    for (int s = 0; s < QG_MAXS; ++s) {
                        if (s >= NS) break;
                        const int hi = (q * QG_MAXS + s) * 2 + (a - 1);
                        const size_t sci = (size_t)T.sc0 + ((size_t)iq * ntq + (size_t)T.wh_col[a - 1]) * QG_MAXS + s;
                        const float r6s = T.qvdw ? r6hc + S.sc_f[sci] : r6hc;
                        const float ir6 = __frcp_rn(r6s);
                        const float Va = S.qwh_A[hi] * ir6 * ir6, Vb = S.qwh_B[hi] * ir6;
                        dv -= lam[s] * ri2 * (12.f * Va - 6.f * Vb) * (r6hc * ir6);
                        if (acc) {
                            const double ir6d = rcp_nr(T.qvdw ? r6hcd + S.sc_d[sci] : r6hcd);
                            evdw.d[s] += S.qwh_Ad[hi] * ir6d * ir6d - S.qwh_Bd[hi] * ir6d;
                        } else if (want) {
                            evdw.k[s].add(Va - Vb);
                        }
                    }
                }
                gx[a] += dv * d.x; gy[a] += dv * d.y; gz[a] += dv * d.z;
                qfx -= dv * d.x; qfy -= dv * d.y; qfz -= dv * d.z;
            }
        }
        q_reduce_store<LG>(sh, iq, on, qfx, qfy, qfz);
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) { gx[a] = group_sum<LG>(gx[a]); gy[a] = group_sum<LG>(gy[a]); gz[a] = group_sum<LG>(gz[a]); }
    if (valid && lane == 0)
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            fx_addf(S.fx + 3 * (a0 + a), gx[a], S.status);
            fx_addf(S.fx + 3 * (a0 + a) + 1, gy[a], S.status);
            fx_addf(S.fx + 3 * (a0 + a) + 2, gz[a], S.status);
        }
    q_flush(S, T, sh);
    if (want) q_energies(S, traj, NS, eel, evdw, acc, EQ_QW_EL, EQ_QW_VDW, sh);
}

// nonbond_qp (src/md.f90:13788-13921) / nonbond_qp_qvdw (14097-14230).
// LG lanes per solute atom of the qp list.
// E as in k_qw.
template <int LG, int E>
__global__ void __launch_bounds__(QG_BLOCK, E == 2 ? 6 : 1) k_qp(DevSys S, const int *satom, EaccSel esel) {
    __shared__ QShared sh;
    const int idx = (blockIdx.x * blockDim.x + threadIdx.x) / LG;
    const int lane = threadIdx.x & (LG - 1);
    const int j = satom[idx];
    const int traj = traj_of_entry(S, j, false);
    const TrajInfo &T = S.traj[traj];
    const bool acc = E != 2 && eacc_on(esel), want = E != 2 && energies_on(esel);
    q_load(S, T, sh);
    const int NS = T.nstates;
    QE eel, evdw;
    eel.zero(); evdw.zero();
    const bool valid = j >= 0 && S.qp_member[j];
    float4 jh = {}, jl = {};
    int tj = 0;
    if (valid) { jh = S.pos[j]; jl = S.poslo[j]; tj = S.atype[j]; }
    // box: the image of the atom that put this group on the list, relative to
    // the Q switching atom (nonbond_qp_box :13960-13969)
    float3 sq = make_float3(0.f, 0.f, 0.f);
    double3 sqd = dzero3();
    if (valid && T.pbc) {
        const int in = S.g_qin[S.agrp[j]];
        sq = box_shift(T, dpos(S.pos[T.qswitch], S.poslo[T.qswitch], S.pos[in], S.poslo[in]));
        if (acc) sqd = box_shift_d(T, S.x, T.qswitch, in);
    }
    float gx = 0.f, gy = 0.f, gz = 0.f;
    const int ntq = T.natyps + T.nqat;
    // per solute atom, loaded once: its LJ row and its 1-4 Q partners
    const int ljrow = T.lj0 + (tj - T.type0) * T.natyps - T.type0;
    const int p14a = valid ? S.qp14_first[j] : 0, p14b = valid ? S.qp14_first[j + 1] : 0;
    for (int iq0 = 0; iq0 < T.nqat; iq0 += LG) {
        const int iq = iq0 + lane;
        const bool on = iq < T.nqat;
        float qfx = 0.f, qfy = 0.f, qfz = 0.f;
        if (valid && on) {
            const int q = T.q0 + iq;
            const int qa = sh.qa[iq];
            const int tq = sh.qt[iq];
            int c = S.ljcod[ljrow + tq];
            for (int k = p14a; k < p14b; ++k)
                if (S.qp14_q[k] == q) c = 3;
            const int qc = c == 2 ? 1 : c;
            const float3 d = f3sub(dpos(sh.qh[iq], sh.ql[iq], jh, jl), sq);
            const float r2 = d.x * d.x + d.y * d.y + d.z * d.z;
            const float ri = rsqrtf(r2), ri2 = ri * ri, r6 = r2 * r2 * r2;
            double rid = 0.0, r6d = 0.0;
            if (acc) { const double r2d = dist2_d(S.x, qa, j, sqd); rid = rsqrt_nr(r2d); r6d = r2d * r2d * r2d; }
            float dv = 0.f;
#pragma unroll
            for (int s = 0; s < QG_MAXS; ++s) {
                if (s >= NS) break;
                float A, B, r6s;
                double Ad = 0, Bd = 0, r6sd = r6d;
                if (T.arith) {
                    // nonbon2_qp (src/md.f90:12221-12376): (a_q + a_j)^6 and b_q b_j,
                    // a_q/b_q of the Q atom's type, or of its state's Q type
                    // (code 2 -> 1) with softcore
                    int ka, kb;
                    const float *ta_, *tb_;
                    const double *ta_d, *tb_d;
                    if (!T.qvdw) { ka = tq * 3 + c - 1; ta_ = S.avdw; tb_ = S.bvdw; ta_d = S.avdw_d; tb_d = S.bvdw_d; r6s = r6; }
                    else {
                        ka = S.qiac[q * QG_MAXS + s] * 3 + qc - 1;
                        ta_ = S.qavdw; tb_ = S.qbvdw; ta_d = S.qavdw_d; tb_d = S.qbvdw_d;
                        r6s = r6 + S.sc_f[(size_t)T.sc0 + ((size_t)iq * ntq + (tj - T.type0)) * QG_MAXS + s];
                        if (acc) r6sd = r6d + S.sc_d[(size_t)T.sc0 + ((size_t)iq * ntq + (tj - T.type0)) * QG_MAXS + s];
                    }
                    kb = tj * 3 + c - 1;
                    float a = ta_[ka] + S.avdw[kb];
                    a = a * a; a = a * a * a;
                    const float b = tb_[ka] * S.bvdw[kb];
                    A = b * a * a; B = 2.f * b * a;
                    if (acc) {
                        double ad = ta_d[ka] + S.avdw_d[kb];
                        ad = ad * ad; ad = ad * ad * ad;
                        const double bd = tb_d[ka] * S.bvdw_d[kb];
                        Ad = bd * ad * ad; Bd = 2.0 * bd * ad;
                    }
                } else if (!T.qvdw) {
                    A = S.avdw[tq * 3 + c - 1] * S.avdw[tj * 3 + c - 1];
                    B = S.bvdw[tq * 3 + c - 1] * S.bvdw[tj * 3 + c - 1];
                    r6s = r6;
                    if (acc) {
                        Ad = S.avdw_d[tq * 3 + c - 1] * S.avdw_d[tj * 3 + c - 1];
                        Bd = S.bvdw_d[tq * 3 + c - 1] * S.bvdw_d[tj * 3 + c - 1];
                    }
                } else {
                    const int qt = S.qiac[q * QG_MAXS + s];
                    const size_t sci = (size_t)T.sc0 + ((size_t)iq * ntq + (tj - T.type0)) * QG_MAXS + s;
                    A = S.qavdw[qt * 3 + qc - 1] * S.avdw[tj * 3 + c - 1];
                    B = S.qbvdw[qt * 3 + qc - 1] * S.bvdw[tj * 3 + c - 1];
                    r6s = r6 + S.sc_f[sci];
                    if (acc) {
                        Ad = S.qavdw_d[qt * 3 + qc - 1] * S.avdw_d[tj * 3 + c - 1];
                        Bd = S.qbvdw_d[qt * 3 + qc - 1] * S.bvdw_d[tj * 3 + c - 1];
                        r6sd = r6d + S.sc_d[sci];
                    }
                }
                float Vel = S.qcrg_f[q * QG_MAXS + s] * jh.w * ri;
                if (c == 3) Vel *= T.el14;
                const float ir6 = __frcp_rn(r6s);
                const float Va = A * ir6 * ir6, Vb = B * ir6;
                dv += T.lambdaf[s] * ri2 * (-Vel - (12.f * Va - 6.f * Vb) * (r6 * ir6));
                if (acc) {
                    double Veld = S.qcrg_d[q * QG_MAXS + s] * S.crg_d[j] * rid;
                    if (c == 3) Veld *= T.el14d;
                    eel.d[s] += Veld;
                    const double ir6d = rcp_nr(r6sd);
                    evdw.d[s] += Ad * ir6d * ir6d - Bd * ir6d;
                } else if (want) {
                    eel.k[s].add(Vel); evdw.k[s].add(Va - Vb);
                }
            }
            gx += dv * d.x; gy += dv * d.y; gz += dv * d.z;
            qfx -= dv * d.x; qfy -= dv * d.y; qfz -= dv * d.z;
        }
        q_reduce_store<LG>(sh, iq, on, qfx, qfy, qfz);
    }
    gx = group_sum<LG>(gx); gy = group_sum<LG>(gy); gz = group_sum<LG>(gz);
    if (valid && lane == 0) {
        fx_addf(S.fx + 3 * j, gx, S.status);
        fx_addf(S.fx + 3 * j + 1, gy, S.status);
        fx_addf(S.fx + 3 * j + 2, gz, S.status);
    }
    q_flush(S, T, sh);
    if (want) q_energies(S, traj, NS, eel, evdw, acc, EQ_QP_EL, EQ_QP_VDW, sh);
}

// Launch shapes (the autotuner's choice, BlockTables::tune): lanes per water
// LW (4/8/16), the register bound of the water kernel (minimum resident
// blocks 1 or 6) and its neighbours per loop iteration (1/2/4); lanes per
// solute atom (4/8/16).  The FP64-energy
// variants (drop-in calls) use 8 lanes.
template <int E, int LW, int MINB, bool BOX>
static void water_fp32(const DevSys &S, const BlockTables &B, LaunchCtx &L, int lrf) {
    const int nb = B.nwgrp * LW / QG_BLOCK;
    if (B.tune.unroll_water == 1) k_nb_water<E, LW, MINB, 1, BOX><<<nb, QG_BLOCK, 0, L.stream>>>(S, B.wgrp, lrf);
    else if (B.tune.unroll_water == 3) k_nb_water<E, LW, MINB, 3, BOX><<<nb, QG_BLOCK, 0, L.stream>>>(S, B.wgrp, lrf);
    else if (B.tune.unroll_water == 4) k_nb_water<E, LW, MINB, 4, BOX><<<nb, QG_BLOCK, 0, L.stream>>>(S, B.wgrp, lrf);
    else k_nb_water<E, LW, MINB, 2, BOX><<<nb, QG_BLOCK, 0, L.stream>>>(S, B.wgrp, lrf);
}
template <int E, bool BOX>
static void water_shapes(const DevSys &S, const BlockTables &B, LaunchCtx &L, int lrf) {
    const bool m6 = B.tune.minb_water == 6;
    switch (B.tune.lw_water) {
    case 4: m6 ? water_fp32<E, 4, 6, BOX>(S, B, L, lrf) : water_fp32<E, 4, 1, BOX>(S, B, L, lrf); break;
    case 16: m6 ? water_fp32<E, 16, 6, BOX>(S, B, L, lrf) : water_fp32<E, 16, 1, BOX>(S, B, L, lrf); break;
    default: m6 ? water_fp32<E, 8, 6, BOX>(S, B, L, lrf) : water_fp32<E, 8, 1, BOX>(S, B, L, lrf); break;
    }
}
template <bool BOX>
static void water_launch(const DevSys &S, const BlockTables &B, LaunchCtx &L, int lrf, int emode) {
    if (emode == QG_PAIR_E_FP64) k_nb_water<1, 8, 1, 2, BOX><<<B.nwgrp * 8 / QG_BLOCK, QG_BLOCK, 0, L.stream>>>(S, B.wgrp, lrf);
    else if (emode == QG_PAIR_E_NONE) water_shapes<2, BOX>(S, B, L, lrf);
    else water_shapes<0, BOX>(S, B, L, lrf);
    if (!B.hlj) return;
    // the LJ of the water hydrogens (arithmetic rule), on the same stream
    const int nb = B.nwgrp * 8 / QG_BLOCK;
    if (emode == QG_PAIR_E_FP64) k_ww_hlj<1, BOX><<<nb, QG_BLOCK, 0, L.stream>>>(S, B.wgrp);
    else if (emode == QG_PAIR_E_NONE) k_ww_hlj<2, BOX><<<nb, QG_BLOCK, 0, L.stream>>>(S, B.wgrp);
    else k_ww_hlj<0, BOX><<<nb, QG_BLOCK, 0, L.stream>>>(S, B.wgrp);
    (*L.nlaunch)++;
}
void launch_nb_water(const DevSys &S, const BlockTables &B, LaunchCtx &L, int lrf, int emode) {
    if (!B.nwgrp) return;
    prof_begin(L, "k_nb_water");
    if (B.pbc) water_launch<true>(S, B, L, lrf, emode);
    else water_launch<false>(S, B, L, lrf, emode);
    prof_end(L);
    (*L.nlaunch)++;
}
template <int E, bool BOX>
static void solute_shapes(const DevSys &S, const BlockTables &B, LaunchCtx &L, int lrf) {
    switch (B.tune.lw_solute) {
    case 4: k_nb_solute<E, 4, BOX><<<B.nsatom * 4 / QG_BLOCK, QG_BLOCK, 0, L.stream>>>(S, B.satom, lrf); break;
    case 16: k_nb_solute<E, 16, BOX><<<B.nsatom * 16 / QG_BLOCK, QG_BLOCK, 0, L.stream>>>(S, B.satom, lrf); break;
    default: k_nb_solute<E, 8, BOX><<<B.nsatom * 8 / QG_BLOCK, QG_BLOCK, 0, L.stream>>>(S, B.satom, lrf); break;
    }
}
template <bool BOX>
static void solute_launch(const DevSys &S, const BlockTables &B, LaunchCtx &L, int lrf, int emode) {
    if (emode == QG_PAIR_E_FP64) k_nb_solute<1, 8, BOX><<<B.nsatom * 8 / QG_BLOCK, QG_BLOCK, 0, L.stream>>>(S, B.satom, lrf);
    else if (emode == QG_PAIR_E_NONE) solute_shapes<2, BOX>(S, B, L, lrf);
    else solute_shapes<0, BOX>(S, B, L, lrf);
}
void launch_nb_solute(const DevSys &S, const BlockTables &B, LaunchCtx &L, int lrf, int emode) {
    if (!B.nsatom) return;
    prof_begin(L, "k_nb_solute");
    if (B.pbc) solute_launch<true>(S, B, L, lrf, emode);
    else solute_launch<false>(S, B, L, lrf, emode);
    prof_end(L);
    (*L.nlaunch)++;
}
// Lanes per item of the Q loops: one per water while each trajectory has
// few Q atoms (the per-item set-up then dominates), more for larger Q sets;
// the qp items (solute atoms) are fewer and always take four.
static int qw_lanes(const BlockTables &B) {
    if (B.tune.lg_qw == 1 || B.tune.lg_qw == 2 || B.tune.lg_qw == 4) return B.tune.lg_qw;
    return B.max_nqat <= 16 ? 1 : (B.max_nqat <= 48 ? 2 : 4);
}

// The shape is tuned on the energy-free form.  The energy form of a recorded
// MD step evaluates the per-state energies in FP64 and is bound by the FP64
// pipe: one lane per water is its fastest shape on the benchmark batch (70 us
// against 81 with four lanes and 93 with two).
template <int E, bool HLJ>
static void qw_shapes_h(const DevSys &S, const BlockTables &B, LaunchCtx &L, EaccSel e) {
    const int lg = E == 2 ? qw_lanes(B) : 1;
    if (lg == 1) k_qw<1, E, HLJ><<<B.nwgrp / QG_BLOCK, QG_BLOCK, 0, L.stream>>>(S, B.wgrp, e);
    else if (lg == 2) k_qw<2, E, HLJ><<<B.nwgrp * 2 / QG_BLOCK, QG_BLOCK, 0, L.stream>>>(S, B.wgrp, e);
    else k_qw<4, E, HLJ><<<B.nwgrp * 4 / QG_BLOCK, QG_BLOCK, 0, L.stream>>>(S, B.wgrp, e);
}
// batches with LJ on some trajectory's water hydrogens take the form that
// adds the Q-H LJ terms
template <int E>
static void qw_shapes(const DevSys &S, const BlockTables &B, LaunchCtx &L, EaccSel e) {
    if (B.hlj) qw_shapes_h<E, true>(S, B, L, e);
    else qw_shapes_h<E, false>(S, B, L, e);
}
// emode QG_PAIR_E_NONE (an MD step whose energies are not recorded) takes the
// energy-free instantiation; every other mode lets esel decide on the device.
void launch_qw(const DevSys &S, const BlockTables &B, LaunchCtx &L, EaccSel e, int emode) {
    if (!B.nwgrp) return;
    prof_begin(L, "k_qw");
    if (emode == QG_PAIR_E_NONE) qw_shapes<2>(S, B, L, e);
    else qw_shapes<0>(S, B, L, e);
    prof_end(L);
    (*L.nlaunch)++;
}
void launch_qp(const DevSys &S, const BlockTables &B, LaunchCtx &L, EaccSel e, int emode) {
    if (!B.nsatom) return;
    prof_begin(L, "k_qp");
    if (emode == QG_PAIR_E_NONE) k_qp<4, 2><<<B.nsatom * 4 / QG_BLOCK, QG_BLOCK, 0, L.stream>>>(S, B.satom, e);
    else k_qp<4, 0><<<B.nsatom * 4 / QG_BLOCK, QG_BLOCK, 0, L.stream>>>(S, B.satom, e);
    prof_end(L);
    (*L.nlaunch)++;
}
