// k_md.cu -- the FP64 update of the master coordinates: Berendsen leap-frog
// (newvel_ber, src/md.f90:6194-6223), SHAKE (shake, 17581-17679), the
// temperature / Berendsen scale (temperature, 6098-6190) and the per-step
// energy summary (pot_energy's assembly, 16186-16218).
#include <math.h>

#include "qgpu_internal.cuh"

#define BOLTZ 0.001986          // src/md.f90:54
#define SHAKE_TOL 0.0001        // src/md.f90:460
#define SHAKE_MAX_ITER 1000     // src/md.f90:461
#ifndef QG_UPD_D_MINB
#define QG_UPD_D_MINB 8         // k_update_d register bound: 8 resident blocks, the grid of the batch in one wave
#endif

// The thermostat's velocity and position update of one atom (md_run
// :6577-6590): Berendsen newvel_ber (v = (v - d winv dv)*Tscale), Langevin
// newvel_lan (v = v*(1 - friction dv) - (d - F_rand) winv dv), Nose-Hoover
// nh_prop scale + newvel_nos; xx = x, x += v dt; with velocity-verlet
// (dv = dt/2) the velocity update is applied again after the position update.
// Consumes and clears the fixed-point gradient.
__global__ void k_integrate(DevSys S) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= S.natom) return;
    const int tr = S.atraj[i];
    const TrajInfo &T = S.traj[tr];
    const TrajState &TS = S.tstate[tr];
    const double ts = (i - T.atom0) < T.nat_solute ? TS.tsd_solute : TS.tsd_solvent;
    const double wi = S.winv[i], dt = T.dt, dvm = T.dvm;
    double rf[3] = {0.0, 0.0, 0.0};
    if (T.thermostat == 1) langevin_force<double>(S, T, TS.rnd, i, rf);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const int k = 3 * i + c;
        const double g = fx_get(S.fx[k]);
        S.fx[k] = 0ull;
        double v = S.v[k];
        if (T.thermostat == 1) v = v * T.lfric - (g - rf[c]) * wi * dvm;
        else if (T.thermostat == 2) v = v * TS.nh_s1 - g * wi * dvm;
        else v = (v - g * wi * dvm) * ts;
        S.xx[k] = S.x[k];
        S.x[k] = S.x[k] + v * dt;
        if (T.integrator == 1) {
            if (T.thermostat == 1) v = v * T.lfric - (g - rf[c]) * wi * dvm;
            else if (T.thermostat == 2) v = v - g * wi * dvm;
            else v = (v - g * wi * dvm) * ts;
        }
        S.v[k] = v;
    }
}

// One thread per molecule with constraints: Gauss-Seidel sweeps until every
// |d0^2 - r^2| < SHAKE_TOL*d0^2, at most SHAKE_MAX_ITER sweeps (then the
// status word reports the failure; the loop is always bounded).
__global__ void k_shake(DevSys S, int traj_filter) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= S.nshk_mol) return;
    const int tr = S.shk_traj[m];
    if (traj_filter >= 0 && tr != traj_filter) return;
    const int c0 = S.shk_first[m], nc = S.shk_first[m + 1] - c0;
    const double *x0 = S.xx;
    double *x = S.x;
    unsigned long long ready = 0ull;
    const unsigned long long all = nc >= 64 ? ~0ull : ((1ull << nc) - 1ull);
    int nits = 0;
    for (;;) {
        for (int c = 0; c < nc; ++c) {
            if (ready & (1ull << c)) continue;
            const int i = S.shk_i[c0 + c], j = S.shk_j[c0 + c];
            const double d2 = S.shk_d2[c0 + c];
            double xij[3], xxij[3];
            for (int a = 0; a < 3; ++a) { xij[a] = x[3 * i + a] - x[3 * j + a]; xxij[a] = x0[3 * i + a] - x0[3 * j + a]; }
            const double xij2 = xij[0] * xij[0] + xij[1] * xij[1] + xij[2] * xij[2];
            const double diff = d2 - xij2;
            if (fabs(diff) < SHAKE_TOL * d2) ready |= (1ull << c);
            const double scp = xij[0] * xxij[0] + xij[1] * xxij[1] + xij[2] * xxij[2];
            const double wi = S.winv[i], wj = S.winv[j];
            // diff / den with a Newton-refined reciprocal (two steps of
            // y <- y (2 - den y) from a float seed reach FP64 precision)
            const double den = 2.0 * scp * (wi + wj);
            double y = (double)__fdividef(1.0f, (float)den);   // seed; refined below
            y = y * (2.0 - den * y);
            y = y * (2.0 - den * y);
            const double corr = diff * y;
            for (int a = 0; a < 3; ++a) {
                x[3 * i + a] += xxij[a] * corr * wi;
                x[3 * j + a] -= xxij[a] * corr * wj;
            }
        }
        nits++;
        if (ready == all) break;
        if (nits >= SHAKE_MAX_ITER) { atomicOr(S.status, ST_SHAKE); atomicCAS(S.status + 1, 0, tr + 1); break; }
    }
    atomicAdd(&S.tstate[tr].shake_iters, nits);
}

// Per-step update of the FP64 path, over the update items (atoms, or whole
// molecules that carry SHAKE constraints):
//   mode 0: kinetic energy + float mirror only (temperature before step 0);
//   mode 2: v = (x - xx)/dt after k_integrate + k_shake (md_run
//           :6596-6597), mirror, Ekin.
// Ekin partials (solute, free solute, solvent, free solvent) per block, as
// float and as int64 fixed point (each atom's 0.5 m v^2 rounded to 2^-32
// kcal/mol, then integer sums: independent of the summation order).
__global__ void __launch_bounds__(QG_BLOCK) k_update(DevSys S, const int *items, int mode) {
    __shared__ double red[4][QG_BLOCK / 32];
    __shared__ long long redq[4][QG_BLOCK / 32];
    const int it = items[blockIdx.x * blockDim.x + threadIdx.x];
    double ek[4] = {0, 0, 0, 0};
    long long ekq[4] = {0, 0, 0, 0};
    if (it >= 0) {
        const bool mol = (it >> 30) & 1;
        const int m = it & 0x3fffffff;
        const int a0 = mol ? S.shk_i[S.shk_first[m]] : m;   // first atom of the item
        const int na = mol ? 3 : 1;
        const int tr = S.atraj[a0];
        const TrajInfo &T = S.traj[tr];
        for (int k = 0; k < na; ++k) {
            const int i = mol ? a0 + k : a0;
            double x[3], v[3], vv = 0;
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                x[a] = S.x[3 * i + a];
                v[a] = S.v[3 * i + a];
                if (mode == 2 && T.nshake_mol > 0) {
                    // v = (x - xx)/dt after SHAKE (md_run :6596-6600), then the
                    // Nose-Hoover second scale
                    v[a] = (x[a] - S.xx[3 * i + a]) * T.inv_dt;
                    if (T.thermostat == 2) v[a] *= S.tstate[tr].nh_s2;
                    S.v[3 * i + a] = v[a];
                }
                vv += v[a] * v[a];
            }
            const double e = 0.5 * S.mass[i] * vv;
            const long long eq = d2fx_chk(e, S.status);
            const bool fr = !S.aexcl[i];
            if ((i - T.atom0) < T.nat_solute) { ek[0] += e; ek[1] += fr ? e : 0; ekq[0] += eq; ekq[1] += fr ? eq : 0; }
            else { ek[2] += e; ek[3] += fr ? e : 0; ekq[2] += eq; ekq[3] += fr ? eq : 0; }
            float4 h, l;
            const double r0 = x[0] - T.origin[0], r1 = x[1] - T.origin[1], r2 = x[2] - T.origin[2];
            h.x = (float)r0; h.y = (float)r1; h.z = (float)r2; h.w = S.pos[i].w;
            l.x = (float)(r0 - (double)h.x); l.y = (float)(r1 - (double)h.y); l.z = (float)(r2 - (double)h.z); l.w = 0.f;
            S.pos[i] = h; S.poslo[i] = l;
            S.velf[i] = make_float4((float)v[0], (float)v[1], (float)v[2], 0.f);
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int k = 0; k < 4; ++k) {
        const double v = warp_sum_d(ek[k]);
        long long q = ekq[k];
        for (int o = 16; o > 0; o >>= 1) q += __shfl_down_sync(0xffffffffu, q, o);
        if (lane == 0) { red[k][warp] = v; redq[k][warp] = q; }
    }
    __syncthreads();
    if (threadIdx.x < 4) {
        double s = 0;
        long long q = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { s += red[threadIdx.x][w]; q += redq[threadIdx.x][w]; }
        S.ekin_part[(size_t)blockIdx.x * 4 + threadIdx.x] = (float)s;
        S.ekin_fx[(size_t)blockIdx.x * 4 + threadIdx.x] = q;
    }
}

// ------------------------------------------------ float-master fused step
// SHAKE of one water in FP32 on relative vectors.  With D_a the displacement
// of atom a in this step and r0 = x_i - x_j the constraint vector at the start
// of the step (a double-float: r0h from the hi parts, r0l from the lo parts),
// the residual of shake (src/md.f90:17620-17650) is
//     diff = d0^2 - |r0 + D_i - D_j|^2 = base - (2 r0 + Dij).Dij,
// base = d0^2 - |r0|^2 formed once per step with two-products / two-sums, so
// the FP32 diff is accurate to about 1e-9 A^2 against the FP64 value and the
// convergence test |diff| < 1e-4 d0^2 takes the same decisions except within
// that distance of the threshold.  The correction follows the reference:
// acor = diff / (2 (winv_i + winv_j) r.r0), x_i += r0 acor winv_i,
// x_j -= r0 acor winv_j, Gauss-Seidel over O-H1, O-H2, H1-H2, constraints
// that met the tolerance once are not revisited, at most SHAKE_MAX_ITER sweeps.
template <int I, int J>
__device__ __forceinline__ void shake_pair_f(float3 (&D)[3], const float3 &r0, const float3 &ua, const float3 &ub,
                                             float base, float S0, float den0, float tol, unsigned &ready, int c) {
    if (ready & (1u << c)) return;
    const float dx = D[I].x - D[J].x, dy = D[I].y - D[J].y, dz = D[I].z - D[J].z;
    const float diff = base - ((2.f * r0.x + dx) * dx + (2.f * r0.y + dy) * dy + (2.f * r0.z + dz) * dz);
    if (fabsf(diff) < tol) ready |= 1u << c;
    const float scp = S0 + (r0.x * dx + r0.y * dy + r0.z * dz);
    const float corr = __fdividef(diff, den0 * scp);
    D[I].x += ua.x * corr; D[I].y += ua.y * corr; D[I].z += ua.z * corr;
    D[J].x -= ub.x * corr; D[J].y -= ub.y * corr; D[J].z -= ub.z * corr;
}

__device__ int shake_water_f(const float4 (&h)[3], const float4 (&l)[3], const float (&w)[3], const float2 (&d2)[3],
                             float3 (&D)[3], bool *fail) {
    const int ci[3] = {0, 0, 1}, cj[3] = {1, 2, 2};
    float3 r0[3], ua[3], ub[3];
    float base[3], S0[3], den0[3], tol[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const int i = ci[c], j = cj[c];
        const float hx = h[i].x - h[j].x, hy = h[i].y - h[j].y, hz = h[i].z - h[j].z;
        const float lx = l[i].x - l[j].x, ly = l[i].y - l[j].y, lz = l[i].z - l[j].z;
        r0[c] = make_float3(hx + lx, hy + ly, hz + lz);
        // |r0h|^2 as an unevaluated sum sh + sl
        float ex, ey, ez, e1, e2;
        const float px = two_prod(hx, hx, ex), py = two_prod(hy, hy, ey), pz = two_prod(hz, hz, ez);
        const float t = two_sum(px, py, e1);
        const float sh = two_sum(t, pz, e2);
        const float sl = ((e1 + e2) + (ex + ey + ez)) + 2.f * (hx * lx + hy * ly + hz * lz);
        base[c] = (d2[c].x - sh) + (d2[c].y - sl);
        S0[c] = sh;
        ua[c] = make_float3(r0[c].x * w[i], r0[c].y * w[i], r0[c].z * w[i]);
        ub[c] = make_float3(r0[c].x * w[j], r0[c].y * w[j], r0[c].z * w[j]);
        den0[c] = 2.f * (w[i] + w[j]);
        tol[c] = (float)SHAKE_TOL * d2[c].x;
    }
    unsigned ready = 0u;
    int nits = 0;
    for (;;) {
        shake_pair_f<0, 1>(D, r0[0], ua[0], ub[0], base[0], S0[0], den0[0], tol[0], ready, 0);
        shake_pair_f<0, 2>(D, r0[1], ua[1], ub[1], base[1], S0[1], den0[1], tol[1], ready, 1);
        shake_pair_f<1, 2>(D, r0[2], ua[2], ub[2], base[2], S0[2], den0[2], tol[2], ready, 2);
        nits++;
        if (ready == 7u) break;
        if (nits >= SHAKE_MAX_ITER) { *fail = true; break; }
    }
    return nits;
}

// x + D on a hi/lo pair, renormalised
__device__ __forceinline__ void hilo_add(float &h, float &l, float d) {
    float e;
    const float s = two_sum(h, d, e);
    h = fast_two_sum(s, l + e, l);
}

// One MD update with the float master state, one thread per atom in blocks
// of QG_UBLK atoms: leap-frog + Berendsen (newvel_ber, src/md.f90:6194-6223)
// per atom; in blocks of 32 waters, warp 0 then runs the SHAKE of one water
// per lane on the displacements held in shared memory; then per atom
// v = (x - xx)/dt (md_run :6596-6597), the hi/lo position update and the
// Ekin partials.  No FP64 arithmetic except the x/v refresh (want_x).
// ekin_only: temperature before the first step (Ekin of the current velf).
__device__ void finalize_traj(const DevSys &S, int tr, int lane, double *v, int do_temp, double *rec,
                              const int *rec_base, int k, int ene_every, int rec_cap);

// fin: FIN_* flags of the step's end (temperature, thermostat state, energy
// record), run by the last block of each trajectory (0: none)
__global__ void __launch_bounds__(QG_UBLK) k_update_f(DevSys S, const int *uatom, const int *ucon,
                                                      const uint8_t *ublk_water, EaccSel esel, int nbcycle,
                                                      int ekin_only, int fin, double *rec, int rec_cap, int ekb0) {
    __shared__ float4 s_h[QG_UBLK], s_l[QG_UBLK];
    __shared__ float s_D[3][QG_UBLK];
    __shared__ float s_w[QG_UBLK];
    __shared__ float red[4][QG_UBLK / 32];
    const int t = threadIdx.x;
    const int a = uatom[blockIdx.x * QG_UBLK + t];
    const bool water_blk = ublk_water[blockIdx.x] != 0;
    const int next = esel.recctl[0] + esel.k + 1;
    const bool want_x = !ekin_only && ((next % nbcycle == 0) ||
                        (esel.mode == EACC_RECORD && esel.ene_every > 0 && next % esel.ene_every == 0));
    // warp 0's SHAKE inputs (first constraint of its water, d0^2), loaded
    // before the atom's own chain of loads so that their latencies overlap
    int c0 = -1;
    float2 d2[3] = {};
    if (water_blk && !ekin_only && t < 32) {
        c0 = ucon[blockIdx.x * QG_UBLK + 3 * t];
        if (c0 >= 0) { d2[0] = S.shk_d2hl[c0]; d2[1] = S.shk_d2hl[c0 + 1]; d2[2] = S.shk_d2hl[c0 + 2]; }
    }
    const int tr = a >= 0 ? S.atraj[a] : -1 - a;
    const TrajInfo &T = S.traj[tr];
    float4 h = make_float4(0, 0, 0, 0), l = h;
    float3 v = make_float3(0, 0, 0), D = v;
    if (a >= 0) {
        const float4 vi = S.velf[a];
        v = make_float3(vi.x, vi.y, vi.z);
        if (!ekin_only) {
            const TrajState &TS = S.tstate[tr];
            h = S.pos[a]; l = S.poslo[a];
            const float w = S.winvf[a], dt = T.dtf;
            const float ts = (a - T.atom0) < T.nat_solute ? TS.tsf_solute : TS.tsf_solvent;
            const float gx = fx_getf(S.fx[3 * a]), gy = fx_getf(S.fx[3 * a + 1]), gz = fx_getf(S.fx[3 * a + 2]);
            S.fx[3 * a] = 0ull; S.fx[3 * a + 1] = 0ull; S.fx[3 * a + 2] = 0ull;
            // the thermostat's update (see k_integrate), in FP32
            const float wdv = w * T.dvmf;
            float rf[3] = {0.f, 0.f, 0.f};
            if (T.thermostat == 1) langevin_force<float>(S, T, TS.rnd, a, rf);
            const float s1 = T.thermostat == 2 ? (float)TS.nh_s1 : 1.f;
            auto kick = [&](float3 u, float fs) {
                if (T.thermostat == 1)
                    return make_float3(u.x * T.lfricf - (gx - rf[0]) * wdv, u.y * T.lfricf - (gy - rf[1]) * wdv,
                                       u.z * T.lfricf - (gz - rf[2]) * wdv);
                if (T.thermostat == 2) return make_float3(u.x * fs - gx * wdv, u.y * fs - gy * wdv, u.z * fs - gz * wdv);
                return make_float3((u.x - gx * wdv) * ts, (u.y - gy * wdv) * ts, (u.z - gz * wdv) * ts);
            };
            v = kick(v, s1);
            D = make_float3(v.x * dt, v.y * dt, v.z * dt);
            if (T.integrator == 1) v = kick(v, 1.f);
            if (water_blk) {
                s_h[t] = h; s_l[t] = l; s_w[t] = w;
                s_D[0][t] = D.x; s_D[1][t] = D.y; s_D[2][t] = D.z;
            }
        }
    }
    if (water_blk && !ekin_only) {
        __syncthreads();
        if (t < 32) {
            int nits = 0;
            if (c0 >= 0) {
                float4 wh[3], wl[3];
                float ww[3];
                float3 wD[3];
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const int q = 3 * t + k;
                    wh[k] = s_h[q]; wl[k] = s_l[q]; ww[k] = s_w[q];
                    wD[k] = make_float3(s_D[0][q], s_D[1][q], s_D[2][q]);
                }
                bool fail = false;
                nits = shake_water_f(wh, wl, ww, d2, wD, &fail);
                if (fail) { atomicOr(S.status, ST_SHAKE); atomicCAS(S.status + 1, 0, tr + 1); }
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const int q = 3 * t + k;
                    s_D[0][q] = wD[k].x; s_D[1][q] = wD[k].y; s_D[2][q] = wD[k].z;
                }
            }
            // a block holds one trajectory: one counter update per block
            for (int o = 16; o > 0; o >>= 1) nits += __shfl_down_sync(0xffffffffu, nits, o);
            if (t == 0 && nits) atomicAdd(&S.tstate[tr].shake_iters, nits);
        }
        __syncthreads();
        if (a >= 0) D = make_float3(s_D[0][t], s_D[1][t], s_D[2][t]);
    }
    float ek[4] = {0.f, 0.f, 0.f, 0.f};
    if (a >= 0) {
        if (!ekin_only) {
            if (T.nshake_mol > 0) {
                v = make_float3(D.x * T.inv_dtf, D.y * T.inv_dtf, D.z * T.inv_dtf);
                if (T.thermostat == 2) {
                    const float s2 = (float)S.tstate[tr].nh_s2;
                    v = make_float3(v.x * s2, v.y * s2, v.z * s2);
                }
            }
            hilo_add(h.x, l.x, D.x);
            hilo_add(h.y, l.y, D.y);
            hilo_add(h.z, l.z, D.z);
            S.pos[a] = h; S.poslo[a] = l;
            S.velf[a] = make_float4(v.x, v.y, v.z, 0.f);
            if (water_blk) { s_h[t] = h; s_l[t] = l; }
            if (want_x) {
                S.x[3 * a] = T.origin[0] + ((double)h.x + (double)l.x);
                S.x[3 * a + 1] = T.origin[1] + ((double)h.y + (double)l.y);
                S.x[3 * a + 2] = T.origin[2] + ((double)h.z + (double)l.z);
                S.v[3 * a] = (double)v.x; S.v[3 * a + 1] = (double)v.y; S.v[3 * a + 2] = (double)v.z;
            }
        }
        const float e = 0.5f * S.massf[a] * (v.x * v.x + v.y * v.y + v.z * v.z);
        const bool fr = !S.aexcl[a];
        if ((a - T.atom0) < T.nat_solute) { ek[0] = e; ek[1] = fr ? e : 0.f; }
        else { ek[2] = e; ek[3] = fr ? e : 0.f; }
    }
    if (water_blk && !ekin_only) {
        // packed water records of the new positions: thread t writes float4
        // t % 3 of the record of water t / 3
        __syncthreads();
        const int w3 = t - t % 3;
        if (ucon[blockIdx.x * QG_UBLK + w3] >= 0) {
            const float4 wh[3] = {s_h[w3], s_h[w3 + 1], s_h[w3 + 2]};
            const float4 wl[3] = {s_l[w3], s_l[w3 + 1], s_l[w3 + 2]};
            S.wrec[uatom[blockIdx.x * QG_UBLK + w3] + t % 3] = wrec_part(wh, wl, t % 3);
        }
    }
    const int lane = t & 31, warp = t >> 5;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float r = warp_sum_f(ek[k]);
        if (lane == 0) red[k][warp] = r;
    }
    __syncthreads();
    if (t < 4) {
        float s = 0.f;
        for (int w = 0; w < QG_UBLK / 32; ++w) s += red[t][w];
        S.ekin_part[((size_t)blockIdx.x + ekb0) * 4 + t] = s;
        __threadfence();
    }
    if (!fin) return;
    // the last block of the trajectory to finish runs the step's end
    __shared__ int s_last;
    __shared__ double s_fin[QG_NE];
    __syncthreads();
    if (t == 0) s_last = atomicAdd(S.fin_cnt + tr, 1) == T.ekin_nblk - 1;
    __syncthreads();
    if (!s_last || t >= 32) return;
    __threadfence();
    finalize_traj(S, tr, t, s_fin, fin, rec, esel.recctl, esel.k, esel.ene_every, rec_cap);
    if (t == 0) S.fin_cnt[tr] = 0;
}

// ------------------------------------------------ FP64-master fused step
// On GB300 an FP64 warp instruction holds its SM sub-partition's FP64 unit
// for about 64-76 cycles whatever lanes are active (1.7 lane-FMAs per clock
// per SM against about 120 in FP32), and the same unit runs the conversions
// between double, float and int64.  The FP64-master step therefore keeps its
// FP64 work to the arithmetic of the reference and converts with integer
// instructions where it can.

// int64 q (|q| < 2^51) as a double: q added to the bits of 1.5*2^52, whose
// ulp is 1, then 1.5*2^52 subtracted (one FP64 add)
__device__ __forceinline__ double ll2d_magic(long long q) {
    return __longlong_as_double(0x4338000000000000LL + q) - 6755399441055744.0;
}
// round-to-nearest-even int64 of v (|v| < 2^51): v + 1.5*2^52 carries the
// rounded integer in its low mantissa bits
__device__ __forceinline__ long long d2ll_magic(double v) {
    return __double_as_longlong(v + 6755399441055744.0) - 0x4338000000000000LL;
}
__device__ __forceinline__ bool magic_range(long long q) {
    return (unsigned long long)(q + (1LL << 51)) < (1ULL << 52);
}

// Round-to-nearest-even float of r from its bits: the 52-bit mantissa is
// rounded at bit 29 (ties to even), the exponent rebiased from 1023 to 127.
// rh receives the float's value as a double.  Values outside the normal float
// range (and zero) take the conversion instruction.
__device__ __forceinline__ float d2f_bits(double r, double &rh) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(r);
    const int e = (int)((b >> 52) & 0x7ffu);
    if (e < 897 || e > 1149) {
        const float f = __double2float_rn(r);
        rh = (double)f;
        return f;
    }
    const unsigned long long rem = b & 0x1fffffffull, half = 0x10000000ull;
    unsigned long long t = b >> 29;                      // sign | exponent | 23 mantissa bits
    t += (rem > half || (rem == half && (t & 1ull))) ? 1ull : 0ull;
    rh = __longlong_as_double((long long)(t << 29));
    const unsigned mag = (unsigned)((t & 0x3ffffffffull) - (896ull << 23));
    return __uint_as_float(mag | (unsigned)((b >> 63) << 31));
}
// hi/lo float pair of r: hi = float(r), lo = float(r - hi) (r - hi is exact;
// it is zero exactly when hi's double has the bits of r, an integer test)
__device__ __forceinline__ void split_hl(double r, float &h, float &l) {
    double rh, rl;
    h = d2f_bits(r, rh);
    const double d = r - rh;
    l = __double_as_longlong(r) == __double_as_longlong(rh) ? 0.f : d2f_bits(d, rl);
}

// 1/den: the PTX approximate FP64 reciprocal (a special-function unit
// instruction) refined by two Newton-Raphson steps y <- y (2 - den y)
__device__ __forceinline__ double rcp_nr(double den) {
    double y;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(den));
    y = y * (2.0 - den * y);
    return y * (2.0 - den * y);
}

// SHAKE of one water in FP64 (shake, src/md.f90:17581-17679), in the
// reference's arithmetic: per constraint xij = x_i - x_j of the current
// positions, diff = d0^2 - |xij|^2, ready once |diff| < SHAKE_TOL d0^2 (the
// correction of that visit is still applied), xxij = xx_i - xx_j of the
// positions before the step, corr = diff / (2 scp (winv_i + winv_j)) with
// scp = xij.xxij, x_i += xxij corr winv_i, x_j -= xxij corr winv_j;
// Gauss-Seidel over O-H1, O-H2, H1-H2; constraints that met the tolerance are
// not revisited; at most SHAKE_MAX_ITER sweeps.  The tolerance test compares
// the bit patterns of |diff| and the (positive) tolerance as integers.  The
// constant factors a = winv / (2 (winv_i + winv_j)) are formed once per water,
// so a visit takes corr winv_i = (diff / scp) a_i: 23 FP64 instructions and
// one reciprocal estimate.  Per-constraint constants (a_i, a_j, d0^2 and the
// tolerance) live in the calling lane's column of cst (shared memory), which
// keeps the registers for the positions.
__device__ __forceinline__ int shake_water_d(double (&x)[3][3], const double (&xx)[3][3], const double (&w)[3],
                                             const double (&d2)[3], double (*cst)[3][32], int lane, bool *fail,
                                             int *visits) {
    double xxij[3][3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const int i = c == 2 ? 1 : 0, j = c == 0 ? 1 : 2;
#pragma unroll
        for (int a = 0; a < 3; ++a) xxij[c][a] = xx[i][a] - xx[j][a];
        const double den0 = 2.0 * (w[i] + w[j]);
        cst[0][c][lane] = w[i] / den0;
        cst[1][c][lane] = w[j] / den0;
        cst[2][c][lane] = d2[c];
        cst[3][c][lane] = SHAKE_TOL * d2[c];
    }
    // (each lane reads back only its own column: no synchronisation)
    // read at every visit (volatile: not hoisted into registers)
    const volatile double (*vc)[3][32] = cst;
    unsigned ready = 0u;
    int nits = 0, nv = 0;
    for (;;) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            if (ready & (1u << c)) continue;
            nv++;
            const int i = c == 2 ? 1 : 0, j = c == 0 ? 1 : 2;
            const double xij0 = x[i][0] - x[j][0], xij1 = x[i][1] - x[j][1], xij2 = x[i][2] - x[j][2];
            const double diff = vc[2][c][lane] - (xij0 * xij0 + xij1 * xij1 + xij2 * xij2);
            if ((__double_as_longlong(diff) & 0x7fffffffffffffffLL) < __double_as_longlong(vc[3][c][lane]))
                ready |= 1u << c;
            const double scp = xij0 * xxij[c][0] + xij1 * xxij[c][1] + xij2 * xxij[c][2];
            const double q = diff * rcp_nr(scp);
            const double ci = q * vc[0][c][lane], cj = q * vc[1][c][lane];
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                x[i][a] += xxij[c][a] * ci;
                x[j][a] -= xxij[c][a] * cj;
            }
        }
        nits++;
        if (ready == 7u) break;
        if (nits >= SHAKE_MAX_ITER) { *fail = true; break; }
    }
    *visits = nv;
    return nits;
}

// One MD step with the FP64 master state, in the fused update's layout (one
// thread per atom in blocks of QG_UBLK: unconstrained atoms first, then
// blocks of 32 waters): per atom the thermostat's FP64 velocity and position
// update of k_integrate (newvel_ber / newvel_lan / newvel_nos, md_run
// :6577-6590); in water blocks warp 0 then runs the FP64 SHAKE of one water
// per lane on the positions held in shared memory; then per atom
// v = (x - xx)/dt (md_run :6596-6600, Nose-Hoover second scale), the FP64
// x/v stores, the float coordinates of the pair kernels (hi/lo of
// x - origin), the packed water records and the Ekin partials (each atom's
// 0.5 m v^2 rounded to 2^-32 kcal/mol, integer sums).  x and v are the
// master: no float state is carried from step to step.  ekin_only: Ekin of
// the current v (temperature before the first step).  fin: the step's end in
// the last block of each trajectory, as in k_update_f.  The per-atom FP64
// work is spread over the block's three warps; the SHAKE of 32 waters is one
// warp's (its FP64 instructions cost the same for any number of active lanes).
__global__ void __launch_bounds__(QG_UBLK, QG_UPD_D_MINB) k_update_d(DevSys S, const int *uatom, const int *ucon,
                                                                     const uint8_t *ublk_water, EaccSel esel,
                                                                     int ekin_only, int fin, double *rec, int rec_cap,
                                                                     int ekb0) {
    __shared__ double s_x[3][QG_UBLK], s_xx[3][QG_UBLK];
    __shared__ float4 s_h[QG_UBLK], s_l[QG_UBLK];
    __shared__ long long red[4][QG_UBLK / 32];
    __shared__ double s_cst[4][3][32];
    const int t = threadIdx.x;
    const int a = uatom[blockIdx.x * QG_UBLK + t];
    const bool water_blk = ublk_water[blockIdx.x] != 0;
    int c0 = -1;
    double d2[3] = {0.0, 0.0, 0.0};
    if (water_blk && !ekin_only && t < 32) {
        c0 = ucon[blockIdx.x * QG_UBLK + 3 * t];
        if (c0 >= 0) { d2[0] = S.shk_d2[c0]; d2[1] = S.shk_d2[c0 + 1]; d2[2] = S.shk_d2[c0 + 2]; }
    }
    const int tr = a >= 0 ? S.atraj[a] : -1 - a;
    const TrajInfo &T = S.traj[tr];
    double x[3] = {0.0, 0.0, 0.0}, xo[3] = {0.0, 0.0, 0.0}, v[3] = {0.0, 0.0, 0.0};
    if (a >= 0) {
#pragma unroll
        for (int c = 0; c < 3; ++c) v[c] = S.v[3 * a + c];
        if (!ekin_only) {
            const TrajState &TS = S.tstate[tr];
            const double wi = S.winv[a];
            const double ts = (a - T.atom0) < T.nat_solute ? TS.tsd_solute : TS.tsd_solvent;
            // gradient (fixed point, 2^-32 units) times winv dv: the 2^-32 is
            // exact, folded into dv
            const double kq = wi * T.dvm_q;
            double rf[3] = {0.0, 0.0, 0.0};
            if (T.thermostat == 1) langevin_force<double>(S, T, TS.rnd, a, rf);
            bool bad = false;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const int k = 3 * a + c;
                xo[c] = S.x[k];
                const long long q = (long long)S.fx[k];
                S.fx[k] = 0ull;
                bad |= !magic_range(q);
                const double gq = ll2d_magic(q);
                double u = v[c];
                if (T.thermostat == 1) u = u * T.lfric - (gq * kq - rf[c] * wi * T.dvm);
                else if (T.thermostat == 2) u = u * TS.nh_s1 - gq * kq;
                else u = (u - gq * kq) * ts;
                x[c] = xo[c] + u * T.dt;
                if (T.integrator == 1) {
                    if (T.thermostat == 1) u = u * T.lfric - (gq * kq - rf[c] * wi * T.dvm);
                    else if (T.thermostat == 2) u = u - gq * kq;
                    else u = (u - gq * kq) * ts;
                }
                v[c] = u;
            }
            if (bad) atomicOr(S.status, ST_FIXED);
            if (water_blk)
#pragma unroll
                for (int c = 0; c < 3; ++c) { s_x[c][t] = x[c]; s_xx[c][t] = xo[c]; }
        }
    }
    if (water_blk && !ekin_only) {
        __syncthreads();
        if (t < 32) {
            int nits = 0, nvis = 0;
            if (c0 >= 0) {
                double wx[3][3], wxx[3][3], ww[3];
                const int o = S.shk_i[c0];
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const int q = 3 * t + k;
#pragma unroll
                    for (int c = 0; c < 3; ++c) { wx[k][c] = s_x[c][q]; wxx[k][c] = s_xx[c][q]; }
                    ww[k] = S.winv[o + k];
                }
                bool failed = false;
                nits = shake_water_d(wx, wxx, ww, d2, s_cst, t, &failed, &nvis);
                if (failed) { atomicOr(S.status, ST_SHAKE); atomicCAS(S.status + 1, 0, tr + 1); }
#pragma unroll
                for (int k = 0; k < 3; ++k)
#pragma unroll
                    for (int c = 0; c < 3; ++c) s_x[c][3 * t + k] = wx[k][c];
            }
            for (int o = 16; o > 0; o >>= 1) {
                nits += __shfl_down_sync(0xffffffffu, nits, o);
                nvis += __shfl_down_sync(0xffffffffu, nvis, o);
            }
            if (t == 0 && nits) { atomicAdd(&S.tstate[tr].shake_iters, nits); atomicAdd(&S.tstate[tr].shake_visits, nvis); }
        }
        __syncthreads();
        // x and xx of this thread's atom come back from shared memory, so
        // that they (and v, formed again below) need no registers during SHAKE
        if (a >= 0)
#pragma unroll
            for (int c = 0; c < 3; ++c) { x[c] = s_x[c][t]; xo[c] = s_xx[c][t]; }
    }
    long long ek[4] = {0, 0, 0, 0};
    if (a >= 0) {
        if (!ekin_only) {
            if (water_blk || T.nshake_mol > 0) {
                const double s2 = T.thermostat == 2 ? S.tstate[tr].nh_s2 : 1.0;
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    v[c] = (x[c] - xo[c]) * T.inv_dt;
                    if (T.thermostat == 2) v[c] *= s2;
                }
            }
            float4 h, l;
            split_hl(x[0] - T.origin[0], h.x, l.x);
            split_hl(x[1] - T.origin[1], h.y, l.y);
            split_hl(x[2] - T.origin[2], h.z, l.z);
            h.w = S.pos[a].w;
            l.w = 0.f;
            S.pos[a] = h; S.poslo[a] = l;
            if (water_blk) { s_h[t] = h; s_l[t] = l; }
#pragma unroll
            for (int c = 0; c < 3; ++c) { S.x[3 * a + c] = x[c]; S.v[3 * a + c] = v[c]; }
        }
        // 0.5 m v^2 in FP64, rounded to 2^-32 kcal/mol: integer sums from here
        const double e = (S.mass[a] * (0.5 * QG_FSCALE)) * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        long long q = d2ll_magic(e);
        // e >= 0: below 2^51 exactly when its bits are (NaN and inf above)
        if (__double_as_longlong(e) >= 0x4320000000000000LL) { atomicOr(S.status, ST_FIXED); q = 0; }
        const bool fr = !S.aexcl[a];
        if ((a - T.atom0) < T.nat_solute) { ek[0] = q; ek[1] = fr ? q : 0; }
        else { ek[2] = q; ek[3] = fr ? q : 0; }
    }
    if (water_blk && !ekin_only) {
        __syncthreads();
        const int w3 = t - t % 3;
        if (ucon[blockIdx.x * QG_UBLK + w3] >= 0) {
            const float4 wh[3] = {s_h[w3], s_h[w3 + 1], s_h[w3 + 2]};
            const float4 wl[3] = {s_l[w3], s_l[w3 + 1], s_l[w3 + 2]};
            S.wrec[uatom[blockIdx.x * QG_UBLK + w3] + t % 3] = wrec_part(wh, wl, t % 3);
        }
    }
    const int lane = t & 31, warp = t >> 5;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        long long r = ek[k];
        for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
        if (lane == 0) red[k][warp] = r;
    }
    __syncthreads();
    if (t < 4) {
        long long sum = 0;
        for (int w = 0; w < QG_UBLK / 32; ++w) sum += red[t][w];
        S.ekin_fx[((size_t)blockIdx.x + ekb0) * 4 + t] = sum;
        __threadfence();
    }
    if (!fin) return;
    __shared__ int s_last;
    __shared__ double s_fin[QG_NE];
    __syncthreads();
    if (t == 0) s_last = atomicAdd(S.fin_cnt + tr, 1) == T.ekin_nblk - 1;
    __syncthreads();
    if (!s_last || t >= 32) return;
    __threadfence();
    finalize_traj(S, tr, t, s_fin, fin, rec, esel.recctl, esel.k, esel.ene_every, rec_cap);
    if (t == 0) S.fin_cnt[tr] = 0;
}

// x = origin + (hi + lo), v = velf: the FP64 view of the float master.
__global__ void k_sync_double(DevSys S) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= S.natom) return;
    const TrajInfo &T = S.traj[S.atraj[i]];
    const float4 h = S.pos[i], l = S.poslo[i], v = S.velf[i];
    S.x[3 * i] = T.origin[0] + ((double)h.x + (double)l.x);
    S.x[3 * i + 1] = T.origin[1] + ((double)h.y + (double)l.y);
    S.x[3 * i + 2] = T.origin[2] + ((double)h.z + (double)l.z);
    S.v[3 * i] = (double)v.x; S.v[3 * i + 1] = (double)v.y; S.v[3 * i + 2] = (double)v.z;
}

// One warp per trajectory: temperature() (optional, every step) and, on the
// steps whose energies are recorded, the energy summary of pot_energy into a
// record row; clears the energy accumulators.  The per-step part is FP32:
// T = Ekin * 2/(Boltz*Ndegf) with the constants formed on the host, the
// Berendsen scale sqrt(1 + dt/tau_T (T0/T - 1)) (src/md.f90:6160-6180).
// FP64 is used for the record rows only.
// nh_prop, src/md.f90:6300-6345: Nose-Hoover chain propagation by dt/2;
// returns the velocity scale s (chain index i = reference i - 1).
__device__ double nh_prop(const TrajInfo &T, double *vnh, double *xnh, double Temp) {
    const int nc = T.nhc;
    if (nc < 1) return 1.0;
    const double dt2 = 0.5 * T.dt, dt4 = 0.5 * dt2, dt8 = 0.5 * dt4, kbT = T.kbT;
    double G[QG_MAXNH];
    double expf = 1.0;
    G[0] = T.Ndegf * BOLTZ * (Temp - T.Temp0) / T.qnh[0];
    for (int i = 1; i < nc; ++i) G[i] = (T.qnh[i - 1] * vnh[i - 1] * vnh[i - 1] - kbT) / T.qnh[i];
    vnh[nc - 1] = vnh[nc - 1] + G[nc - 1] * dt4;
    xnh[nc - 1] = xnh[nc - 1] + vnh[nc - 1] * dt2;
    for (int i = nc - 2; i >= 0; --i) {
        expf = exp(-dt8 * vnh[i + 1]);
        vnh[i] = (vnh[i] * expf + G[i] * dt4) * expf;
        xnh[i] = xnh[i] + vnh[i] * dt2;
    }
    const double sc = exp(-vnh[0] * dt2);
    G[0] = T.Ndegf * BOLTZ * (sc * sc * Temp - T.Temp0) / T.qnh[0];
    vnh[0] = (vnh[0] * expf + G[0] * dt4) * expf;
    for (int i = 1; i < nc - 1; ++i) {
        expf = exp(-dt8 * vnh[i + 1]);
        G[i] = (T.qnh[i - 1] * vnh[i - 1] * vnh[i - 1] - kbT) / T.qnh[i];
        vnh[i] = (vnh[i] * expf + G[i] * dt4) * expf;
    }
    if (nc > 1) {
        G[nc - 1] = (T.qnh[nc - 2] * vnh[nc - 2] * vnh[nc - 2] - kbT) / T.qnh[nc - 1];
        vnh[nc - 1] = vnh[nc - 1] + G[nc - 1] * dt4;
    }
    return sc;
}

// The end of a step for trajectory tr, run by one warp (lane = 0..31; v a
// shared QG_NE scratch): energy accumulators into the record row on recorded
// steps (and cleared), FEP sums, temperature and thermostat state.
// do_temp: FIN_* flags.  Ekin partials and accumulators are read with
// ld.global.cg: in the fused update the last block of a trajectory runs this
// after the other blocks' writes (made visible by __threadfence).
__device__ void finalize_traj(const DevSys &S, int tr, int lane, double *v, int do_temp, double *rec,
                              const int *rec_base, int k, int ene_every, int rec_cap) {
    const TrajInfo &T = S.traj[tr];
    TrajState &TS = S.tstate[tr];
    unsigned long long *ea = S.eacc + (size_t)tr * QG_NE;
    int row = -1;
    const int fstep = rec_base[0] + k;
    const bool rec_step = rec && ene_every > 0 && fstep % ene_every == 0;
    if (rec_step) {
        row = fstep / ene_every - rec_base[1];
        if (row >= rec_cap) row = -1;
    }
    // FEP frames: qdyn writes energy frames at nonzero recorded steps only
    const bool fep = rec_step && T.fep_on && fstep > 0;
    for (int s = lane; s < QG_NE; s += 32) {
        if (row >= 0 || fep) v[s] = fx_get(__ldcg(ea + s));
        ea[s] = 0ull;
    }
    __syncwarp();
    if (fep && lane == 0 && ++TS.fep_n > T.fep_nskip) {
        // qfep Part 1 (src/qfep.f90:609-655): dv = veff2 - veff1 in qfep's
        // operation order, sums in frame order; V_s = EQ(s)%total
        double *A = S.fep_acc + (size_t)tr * QG_NFEP;
        double ve = 0.0, vf = 0.0, vr = 0.0;
        for (int s = 0; s < T.nstates; ++s) {
            const double *w = v + EA_Q0 + EQ_N * s;
            const double Vs = w[EQ_B] + w[EQ_A] + w[EQ_T] + w[EQ_I] + (w[EQ_QQ_EL] + w[EQ_QP_EL] + w[EQ_QW_EL]) +
                              (w[EQ_QQ_VDW] + w[EQ_QP_VDW] + w[EQ_QW_VDW]) + w[EQ_RST];
            ve += T.lambda[s] * Vs;
            vf += T.fep_lamf[s] * Vs;
            vr += T.fep_lamr[s] * Vs;
        }
        A[0] += 1.0;
        if (T.fep_has_f) {
            const double dv = vf - ve;
            A[1] += exp(-dv / T.fep_kT); A[2] += dv; A[3] += dv * dv; A[4] += dv * dv * dv;
        }
        if (T.fep_has_r) {
            const double dv = vr - ve;
            A[5] += exp(-dv / T.fep_kT); A[6] += dv; A[7] += dv * dv; A[8] += dv * dv * dv;
        }
    }
    if (do_temp & FIN_EK64) {
        // temperature (src/md.f90:6098-6190) in FP64 from the int64 partials:
        // exact integer sums, then the reference's operation order
        long long p[4] = {0, 0, 0, 0};
        const long long *ep = S.ekin_fx + 4 * (size_t)T.ekin_blk0;
        for (int b = lane; b < T.ekin_nblk; b += 32)
#pragma unroll
            for (int k = 0; k < 4; ++k) p[k] += __ldcg(ep + 4 * b + k);
#pragma unroll
        for (int k = 0; k < 4; ++k)
            for (int o = 16; o > 0; o >>= 1) p[k] += __shfl_down_sync(0xffffffffu, p[k], o);
        if (lane == 0) {
            const double e_su = fx_get((unsigned long long)p[0]), f_su = fx_get((unsigned long long)p[1]);
            const double e_sv = fx_get((unsigned long long)p[2]), f_sv = fx_get((unsigned long long)p[3]);
            const double Ekin = e_su + e_sv;
            const double Temp = T.Ndegf > 0 ? 2.0 * Ekin / BOLTZ / (double)T.Ndegf : 0.0;
            const double Tfree = T.Ndegfree > 0 ? 2.0 * (f_sv + f_su) / BOLTZ / (double)T.Ndegfree : 0.0;
            double Tfsu = f_su, Tfsv = f_sv;
            if (T.detail_temps) {
                Tfsu = T.Ndegfree_solute > 0 ? 2.0 * Tfsu / BOLTZ / (double)T.Ndegfree_solute : 0.0;
                Tfsv = T.Ndegfree_solvent > 0 ? 2.0 * Tfsv / BOLTZ / (double)T.Ndegfree_solvent : 0.0;
            }
            double ts = TS.tsd_solvent, tu = TS.tsd_solute;
            if (T.thermostat != 0) {
                ts = 1.0; tu = 1.0;
            } else if (T.separate_scaling) {
                if (Tfsv != 0.0) ts = T.Temp0 / Tfsv - 1.0;
                ts = sqrt(1.0 + T.dt_taud * ts);
                if (Tfsu != 0.0) tu = T.Temp0 / Tfsu - 1.0;
                tu = sqrt(1.0 + T.dt_taud * tu);
            } else {
                if (Tfree != 0.0) ts = T.Temp0 / Tfree - 1.0;
                ts = sqrt(1.0 + T.dt_taud * ts);
                tu = ts;
            }
            TS.Ekin_d = Ekin; TS.Temp_d = Temp; TS.Tfree_d = Tfree;
            TS.tsd_solute = tu; TS.tsd_solvent = ts;
            TS.Ekin = (float)Ekin; TS.Temp = (float)Temp; TS.Tfree = (float)Tfree;
            TS.tsf_solute = (float)tu; TS.tsf_solvent = (float)ts;
            TS.wshiftf = T.fk_wsphere != 0.0 ? (float)sqrt(BOLTZ * Tfree / T.fk_wsphere) : 0.f;
            if (Temp != Temp) atomicOr(S.status, ST_NAN);
            if (T.thermostat == 1 && (do_temp & FIN_STEP))
                TS.rnd = (unsigned)((T.lcgA * TS.rnd + T.lcgC) % QG_LCG_M);
            if (T.thermostat == 2 && (do_temp & FIN_NH)) {
                double *vnh = S.nh_state + (size_t)tr * 2 * QG_MAXNH, *xnh = vnh + QG_MAXNH;
                TS.nh_s1 = nh_prop(T, vnh, xnh, Temp);
                TS.nh_s2 = T.nshake_mol > 0 ? nh_prop(T, vnh, xnh, Temp) : 1.0;
            }
        }
    } else if (do_temp) {
        // the four partials of a block are one float4 (slots 4 b .. 4 b + 3)
        float4 p = make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 *ep = reinterpret_cast<const float4 *>(S.ekin_part) + T.ekin_blk0;
        for (int b = lane; b < T.ekin_nblk; b += 32) {
            const float4 q = __ldcg(ep + b);
            p.x += q.x; p.y += q.y; p.z += q.z; p.w += q.w;
        }
        const float e4[4] = {warp_sum_f(p.x), warp_sum_f(p.y), warp_sum_f(p.z), warp_sum_f(p.w)};
        if (lane == 0) {
            float Tfsu = e4[1], Tfsv = e4[3];
            const float Ekin = e4[0] + e4[2];
            const float Temp = Ekin * T.cT, Tfree = (e4[1] + e4[3]) * T.cTfree;
            if (T.detail_temps) { Tfsu *= T.cTfsu; Tfsv *= T.cTfsv; }
            float ts = TS.tsf_solvent, tu = TS.tsf_solute;
            if (T.thermostat != 0) {
                ts = 1.f; tu = 1.f;   // only the Berendsen thermostat scales (md.f90:6166)
            } else if (T.separate_scaling) {
                if (Tfsv != 0.f) ts = T.Temp0f / Tfsv - 1.f;
                ts = sqrtf(1.f + T.dt_tau * ts);
                if (Tfsu != 0.f) tu = T.Temp0f / Tfsu - 1.f;
                tu = sqrtf(1.f + T.dt_tau * tu);
            } else {
                if (Tfree != 0.f) ts = T.Temp0f / Tfree - 1.f;
                ts = sqrtf(1.f + T.dt_tau * ts);
                tu = ts;
            }
            TS.Ekin = Ekin; TS.Temp = Temp; TS.Tfree = Tfree;
            TS.tsf_solute = tu; TS.tsf_solvent = ts;
            TS.Ekin_d = Ekin; TS.Temp_d = Temp; TS.Tfree_d = Tfree;
            TS.tsd_solute = tu; TS.tsd_solvent = ts;
            TS.wshiftf = T.fk_wspheref != 0.f ? sqrtf(0.001986f * Tfree / T.fk_wspheref) : 0.f;
            if (Temp != Temp) atomicOr(S.status, ST_NAN);
            if (T.thermostat == 1 && (do_temp & FIN_STEP))
                TS.rnd = (unsigned)((T.lcgA * TS.rnd + T.lcgC) % QG_LCG_M);
            if (T.thermostat == 2 && (do_temp & FIN_NH)) {
                // the two nh_prop calls of the next step (before the update and
                // after SHAKE, md_run :6584-6600) both read this temperature
                double *vnh = S.nh_state + (size_t)tr * 2 * QG_MAXNH, *xnh = vnh + QG_MAXNH;
                TS.nh_s1 = nh_prop(T, vnh, xnh, (double)Temp);
                TS.nh_s2 = T.nshake_mol > 0 ? nh_prop(T, vnh, xnh, (double)Temp) : 1.0;
            }
        }
    }
    __syncwarp();
    if (lane != 0 || row < 0) return;
    double *R = rec + ((size_t)row * S.ntraj + tr) * QG_REC;
    // Q energies per state
    double qb = 0, qa = 0, qt = 0, qi = 0, qxe = 0, qxv = 0, qr = 0;
    for (int s = 0; s < QG_MAXS; ++s) {
        double *q = R + QG_REC_EQ + 15 * s;
        for (int c = 0; c < 15; ++c) q[c] = 0;
        if (s >= T.nstates) continue;
        const double *w = v + EA_Q0 + EQ_N * s;
        const double lam = T.lambda[s];
        q[0] = lam;
        q[1] = w[EQ_B]; q[2] = w[EQ_A]; q[3] = w[EQ_T]; q[4] = w[EQ_I];
        q[5] = w[EQ_QQ_EL]; q[6] = w[EQ_QQ_VDW]; q[7] = w[EQ_QP_EL]; q[8] = w[EQ_QP_VDW];
        q[9] = w[EQ_QW_EL]; q[10] = w[EQ_QW_VDW];
        q[11] = q[5] + q[7] + q[9];
        q[12] = q[6] + q[8] + q[10];
        q[13] = w[EQ_RST];
        q[14] = q[1] + q[2] + q[3] + q[4] + q[11] + q[12] + q[13];
        qb += q[1] * lam; qa += q[2] * lam; qt += q[3] * lam; qi += q[4] * lam;
        qxe += q[11] * lam; qxv += q[12] * lam; qr += q[13] * lam;
    }
    double *E = R + QG_REC_E;
    // field order of qgpu_energies
    E[2] = v[EA_LRF];
    E[3] = v[EA_P_BOND]; E[4] = v[EA_P_ANG]; E[5] = v[EA_P_TOR]; E[6] = v[EA_P_IMP];
    E[7] = v[EA_W_BOND]; E[8] = v[EA_W_ANG]; E[9] = v[EA_W_TOR]; E[10] = v[EA_W_IMP];
    E[11] = qb; E[12] = qa; E[13] = qt; E[14] = qi;
    E[15] = v[EA_PP_EL]; E[16] = v[EA_PP_VDW]; E[17] = v[EA_PW_EL]; E[18] = v[EA_PW_VDW];
    E[19] = v[EA_WW_EL]; E[20] = v[EA_WW_VDW]; E[21] = qxe; E[22] = qxv;
    // the per-state restraints enter the protein restraint lambda-weighted (pot_energy)
    E[24] = v[EA_RST_FIX]; E[25] = v[EA_RST_SHELL]; E[26] = v[EA_RST_PROT] + qr; E[27] = v[EA_RST_RAD];
    E[28] = v[EA_RST_WPOL];
    E[23] = E[24] + E[25] + E[26] + E[27] + E[28];
    E[0] = E[3] + E[7] + E[4] + E[8] + E[5] + E[6] + E[15] + E[16] + E[17] + E[18] + E[19] + E[20] + E[11] + E[12] +
           E[13] + E[14] + E[21] + E[22] + E[23] + E[2];
    E[1] = TS.Ekin_d;
    R[QG_REC_T] = TS.Temp_d;
    R[QG_REC_T + 1] = TS.Tfree_d;
    for (int c = 0; c < 2 * QG_MAXOD; ++c) R[QG_REC_OD + c] = S.od_out[(size_t)tr * QG_MAXOD * 2 + c];
}

// One warp per trajectory (the FP64 path, temperature before the first step,
// drop-in energy calls).
__global__ void k_finalize(DevSys S, int do_temp, double *rec, const int *rec_base, int k, int ene_every, int rec_cap) {
    __shared__ double v[QG_NE];
    finalize_traj(S, blockIdx.x, threadIdx.x, v, do_temp, rec, rec_base, k, ene_every, rec_cap);
}

__global__ void k_tick(int *rec_base, int n) {
    if (threadIdx.x == 0 && blockIdx.x == 0) *rec_base += n;
}

// Writes the record control words from launch arguments: a copy from pageable
// host memory would make the host wait for the stream.
__global__ void k_set_ctl(int *ctl, int n, int a, int b) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        ctl[0] = a;
        if (n > 1) ctl[1] = b;
    }
}

__global__ void k_grad_to_double(DevSys S, double *out, int atom0, int n3) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n3) return;
    out[k] = fx_get(S.fx[3 * atom0 + k]);
}

static inline int nblk(int n, int b) { return (n + b - 1) / b; }

void launch_integrate(const DevSys &S, const BlockTables &B, LaunchCtx &L) {
    prof_begin(L, "k_integrate");
    k_integrate<<<nblk(S.natom, 256), 256, 0, L.stream>>>(S);
    prof_end(L);
    (*L.nlaunch)++;
}
void launch_shake(const DevSys &S, const BlockTables &B, LaunchCtx &L, int traj_filter) {
    if (!S.nshk_mol) return;
    prof_begin(L, "k_shake");
    k_shake<<<nblk(S.nshk_mol, 128), 128, 0, L.stream>>>(S, traj_filter);
    prof_end(L);
    (*L.nlaunch)++;
}
void launch_update(const DevSys &S, const BlockTables &B, LaunchCtx &L, int mode) {
    prof_begin(L, "k_update");
    k_update<<<B.nuitem / QG_BLOCK, QG_BLOCK, 0, L.stream>>>(S, B.uitem, mode);
    prof_end(L);
    (*L.nlaunch)++;
}
void launch_update_f(const DevSys &S, const BlockTables &B, LaunchCtx &L, EaccSel e, int nbcycle, int ekin_only,
                     int fin, double *rec, int rec_cap) {
    prof_begin(L, "k_update_f");
    k_update_f<<<B.nuatom / QG_UBLK, QG_UBLK, 0, L.stream>>>(S, B.uatom, B.ucon, B.ublk_water, e, nbcycle, ekin_only,
                                                             fin, rec, rec_cap, B.ublk0);
    prof_end(L);
    (*L.nlaunch)++;
}
void launch_update_d(const DevSys &S, const BlockTables &B, LaunchCtx &L, EaccSel e, int ekin_only, int fin,
                     double *rec, int rec_cap) {
    prof_begin(L, "k_update_d");
    k_update_d<<<B.nuatom / QG_UBLK, QG_UBLK, 0, L.stream>>>(S, B.uatom, B.ucon, B.ublk_water, e, ekin_only, fin, rec,
                                                             rec_cap, B.ublk0);
    prof_end(L);
    (*L.nlaunch)++;
}
void launch_sync_double(const DevSys &S, const BlockTables &B, LaunchCtx &L) {
    prof_begin(L, "k_sync_double");
    k_sync_double<<<nblk(S.natom, 256), 256, 0, L.stream>>>(S);
    prof_end(L);
    (*L.nlaunch)++;
}
void launch_finalize(const DevSys &S, LaunchCtx &L, int do_temperature, double *rec, const int *rec_base, int k,
                     int ene_every, int rec_cap) {
    prof_begin(L, "k_finalize");
    k_finalize<<<S.ntraj, 32, 0, L.stream>>>(S, do_temperature, rec, rec_base, k, ene_every, rec_cap);
    prof_end(L);
    (*L.nlaunch)++;
}
void launch_tick(LaunchCtx &L, int *rec_base, int n) {
    prof_begin(L, "k_tick");
    k_tick<<<1, 32, 0, L.stream>>>(rec_base, n);
    prof_end(L);
    (*L.nlaunch)++;
}
void launch_set_ctl(LaunchCtx &L, int *ctl, int n, int a, int b) {
    prof_begin(L, "k_set_ctl");
    k_set_ctl<<<1, 32, 0, L.stream>>>(ctl, n, a, b);
    prof_end(L);
    (*L.nlaunch)++;
}
void launch_grad_to_double(const DevSys &S, LaunchCtx &L, double *out, int atom0, int natom) {
    prof_begin(L, "k_grad_to_double");
    k_grad_to_double<<<nblk(3 * natom, 256), 256, 0, L.stream>>>(S, out, atom0, 3 * natom);
    prof_end(L);
    (*L.nlaunch)++;
}

// FP32 FMA throughput probe: 8 independent FMA chains per thread.
__global__ void k_fma_peak(float *out, int iters, float a, float b) {
    float r0 = threadIdx.x, r1 = r0 + 1, r2 = r0 + 2, r3 = r0 + 3, r4 = r0 + 4, r5 = r0 + 5, r6 = r0 + 6, r7 = r0 + 7;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            r0 = fmaf(r0, a, b); r1 = fmaf(r1, a, b); r2 = fmaf(r2, a, b); r3 = fmaf(r3, a, b);
            r4 = fmaf(r4, a, b); r5 = fmaf(r5, a, b); r6 = fmaf(r6, a, b); r7 = fmaf(r7, a, b);
        }
    }
    const float s = r0 + r1 + r2 + r3 + r4 + r5 + r6 + r7;
    if (s == 12345.678f) out[0] = s;   // keeps the chains live
}

// FP64 FMA throughput probe: 8 independent DFMA chains per thread.
__global__ void k_dfma_peak(double *out, int iters, double a, double b) {
    double r0 = threadIdx.x, r1 = r0 + 1, r2 = r0 + 2, r3 = r0 + 3, r4 = r0 + 4, r5 = r0 + 5, r6 = r0 + 6, r7 = r0 + 7;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            r0 = fma(r0, a, b); r1 = fma(r1, a, b); r2 = fma(r2, a, b); r3 = fma(r3, a, b);
            r4 = fma(r4, a, b); r5 = fma(r5, a, b); r6 = fma(r6, a, b); r7 = fma(r7, a, b);
        }
    }
    const double s = r0 + r1 + r2 + r3 + r4 + r5 + r6 + r7;
    if (s == 12345.678) out[0] = s;   // keeps the chains live
}

extern "C" int qgpu_fp64_peak(double *tflops) {
    if (!tflops) return 1;
    int dev = 0, nsm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 2;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    double *out = nullptr;
    if (cudaMalloc(&out, sizeof(double)) != cudaSuccess) return 2;
    const int threads = 256, blocks = nsm * 2, iters = 64;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    k_dfma_peak<<<blocks, threads>>>(out, 4, 0.999, 0.001);   // warm-up
    cudaEventRecord(a);
    k_dfma_peak<<<blocks, threads>>>(out, iters, 0.999, 0.001);
    cudaEventRecord(b);
    cudaEventSynchronize(b);
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    const double flops = 2.0 * 8 * 4 * (double)iters * threads * blocks;
    *tflops = flops / (ms * 1e-3) / 1e12;
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(out);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

extern "C" int qgpu_fp32_peak(double *tflops) {
    if (!tflops) return 1;
    int dev = 0, nsm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 2;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    float *out = nullptr;
    if (cudaMalloc(&out, sizeof(float)) != cudaSuccess) return 2;
    const int threads = 256, blocks = nsm * 8, iters = 2048;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    k_fma_peak<<<blocks, threads>>>(out, 64, 0.999f, 0.001f);   // warm-up
    cudaEventRecord(a);
    k_fma_peak<<<blocks, threads>>>(out, iters, 0.999f, 0.001f);
    cudaEventRecord(b);
    cudaEventSynchronize(b);
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    const double flops = 2.0 * 8 * 16 * (double)iters * threads * blocks;
    *tflops = flops / (ms * 1e-3) / 1e12;
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(out);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}
