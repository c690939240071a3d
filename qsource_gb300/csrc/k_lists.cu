// k_lists.cu -- charge-group centres, the fused pair-list + LRF scan, and the
// Q-atom list membership (make_pair_lists, src/md.f90:5985-6071).
#include "qgpu_internal.cuh"

// float mirror of the FP64 coordinates: hi = float(x - origin),
// lo = float((x - origin) - hi), w = scaled charge; float velocities.
__global__ void k_mirror(DevSys S) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= S.natom) return;
    const TrajInfo &T = S.traj[S.atraj[i]];
    float4 h, l;
    double r0 = S.x[3 * i] - T.origin[0], r1 = S.x[3 * i + 1] - T.origin[1], r2 = S.x[3 * i + 2] - T.origin[2];
    h.x = (float)r0; h.y = (float)r1; h.z = (float)r2; h.w = S.pos[i].w;
    l.x = (float)(r0 - (double)h.x); l.y = (float)(r1 - (double)h.y); l.z = (float)(r2 - (double)h.z); l.w = 0.f;
    S.pos[i] = h;
    S.poslo[i] = l;
    S.velf[i] = make_float4((float)S.v[3 * i], (float)S.v[3 * i + 1], (float)S.v[3 * i + 2], 0.f);
}

// k_mirror over atoms [a0, a0 + n) of one trajectory, with the packed
// records of its waters (each water's O thread forms them from x).
__global__ void k_mirror_range(DevSys S, int a0, int n) {
    const int i = a0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a0 + n) return;
    const TrajInfo &T = S.traj[S.atraj[i]];
    float4 h[3], l[3];
    const int na = S.g_kind[S.agrp[i]] && S.g_atoms[S.g_start[S.agrp[i]]] == i ? 3 : 1;
    for (int k = 0; k < na; ++k) {
        const int a = i + k;
        const double r0 = S.x[3 * a] - T.origin[0], r1 = S.x[3 * a + 1] - T.origin[1], r2 = S.x[3 * a + 2] - T.origin[2];
        h[k].x = (float)r0; h[k].y = (float)r1; h[k].z = (float)r2; h[k].w = S.pos[a].w;
        l[k].x = (float)(r0 - (double)h[k].x); l[k].y = (float)(r1 - (double)h[k].y); l[k].z = (float)(r2 - (double)h[k].z);
        l[k].w = 0.f;
    }
    S.pos[i] = h[0];
    S.poslo[i] = l[0];
    S.velf[i] = make_float4((float)S.v[3 * i], (float)S.v[3 * i + 1], (float)S.v[3 * i + 2], 0.f);
    if (na == 3) put_wrec(S.wrec + i, h, l);
}

__global__ void k_wrec(DevSys S, const int *wgrp, int n) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int w = wgrp[k];
    if (w < 0) return;
    const int a0 = S.g_atoms[S.g_start[w]];
    float4 h[3], l[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) { h[a] = S.pos[a0 + a]; l[a] = S.poslo[a0 + a]; }
    put_wrec(S.wrec + a0, h, l);
}

// cgp_centers, src/md.f90:2253-2288: mean of the member coordinates (FP64),
// and its float offset from the trajectory origin for the per-step kernels.
__global__ void k_centers(DevSys S, int gb, int gn) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= gn) return;
    const int g = gb + k;
    double c0 = 0, c1 = 0, c2 = 0;
    int a0 = S.g_start[g], a1 = S.g_start[g + 1];
    for (int k = a0; k < a1; ++k) {
        int a = S.g_atoms[k];
        c0 += S.x[3 * a]; c1 += S.x[3 * a + 1]; c2 += S.x[3 * a + 2];
    }
    double n = (double)(a1 - a0);
    const double m0 = c0 / n, m1 = c1 / n, m2 = c2 / n;
    S.g_cent[3 * g] = m0; S.g_cent[3 * g + 1] = m1; S.g_cent[3 * g + 2] = m2;
    const TrajInfo &T = S.traj[S.g_traj[g]];
    // .w: distance from the switch atom to the farthest member (rounded up),
    // the bound of the any-atom cut-off test (nb*lis2*)
    const int sw = S.g_switch[g];
    double e2 = 0.0;
    for (int k = a0; k < a1; ++k) {
        const int a = S.g_atoms[k];
        const double dx = S.x[3 * a] - S.x[3 * sw], dy = S.x[3 * a + 1] - S.x[3 * sw + 1], dz = S.x[3 * a + 2] - S.x[3 * sw + 2];
        e2 = fmax(e2, dx * dx + dy * dy + dz * dz);
    }
    const float ext = (float)sqrt(e2) * (1.f + 1e-5f) + 1e-4f;
    S.g_centf[g] = make_float4((float)(m0 - T.origin[0]), (float)(m1 - T.origin[1]), (float)(m2 - T.origin[2]), ext);
}

// Cut-off decision of the list builders (nbpplist_lrf :8083-8090,
// nbpwlist_lrf :9382-9388, nbwwlist_lrf :10982-10986): FP32 prefilter on the
// hi/lo representative-atom distance, exact FP64 recheck inside a 1e-5 band
// so the decision equals the FP64 test `r2 <= rc**2` bit for bit.
__device__ __forceinline__ bool within(float d2, float rc2, double drc2, const double *x, int a, int b) {
    if (d2 < rc2 * (1.f - 1e-5f)) return true;
    if (d2 > rc2 * (1.f + 1e-5f)) return false;
    return dist2_exact(x, a, b) <= drc2;
}
// the same for a minimum-image distance in a periodic box
__device__ __forceinline__ bool within_box(float d2, float rc2, double drc2, const double *x, int a, int b,
                                           const TrajInfo &T) {
    if (d2 < rc2 * (1.f - 1e-5f)) return true;
    if (d2 > rc2 * (1.f + 1e-5f)) return false;
    return dist2_exact_box(x, a, b, T) <= drc2;
}
// the same with a 1e-4 band, for distances from hi-only float coordinates
__device__ __forceinline__ bool within_hi(float d2, float rc2, double drc2, const double *x, int a, int b) {
    if (d2 < rc2 * (1.f - 1e-4f)) return true;
    if (d2 > rc2 * (1.f + 1e-4f)) return false;
    return dist2_exact(x, a, b) <= drc2;
}
__device__ __forceinline__ float d2hi(const float4 a, const float4 b) {
    const float dx = b.x - a.x, dy = b.y - a.y, dz = b.z - a.z;
    return dx * dx + dy * dy + dz * dz;
}
// the minimum-image forms of the two, for an atom pair in a periodic box
__device__ __forceinline__ float d2hi_box(const float4 a, const float4 b, const TrajInfo &T) {
    float3 d = make_float3(b.x - a.x, b.y - a.y, b.z - a.z);
    d = f3sub(d, box_shift(T, d));
    return d.x * d.x + d.y * d.y + d.z * d.z;
}
__device__ __forceinline__ bool within_hi_box(float d2, float rc2, double drc2, const double *x, int a, int b,
                                              const TrajInfo &T) {
    if (d2 < rc2 * (1.f - 1e-4f)) return true;
    if (d2 > rc2 * (1.f + 1e-4f)) return false;
    return dist2_exact_box(x, a, b, T) <= drc2;
}

// lrf_update (src/md.f90:5896-5981) of one source atom p (charge in .w) at
// the target centre c: the 24 symmetric FP32 sums of the multipole expansion.
__device__ __forceinline__ void lrf_acc(float (&acc)[QG_NLRF], const float4 p, float cx, float cy, float cz) {
    const float dx = p.x - cx, dy = p.y - cy, dz = p.z - cz;
    const float r2 = dx * dx + dy * dy + dz * dz;
    const float ri = rsqrtf(r2), ri2 = ri * ri;
    const float f0 = p.w * ri * ri2;
    const float f1 = 3.f * f0 * ri2;
    const float f2 = -f1 * ri2;
    acc[0] += p.w * ri;
    acc[1] += f0;
    acc[2] += f0 * dx; acc[3] += f0 * dy; acc[4] += f0 * dz;
    const float ux = f1 * dx, uy = f1 * dy, uz = f1 * dz;
    acc[5] += ux; acc[6] += uy; acc[7] += uz;
    acc[8] += ux * dx; acc[9] += uy * dy; acc[10] += uz * dz;
    acc[11] += ux * dy; acc[12] += ux * dz; acc[13] += uy * dz;
    const float vx = f2 * dx, vy = f2 * dy, vz = f2 * dz;
    const float wxx = vx * dx, wyy = vy * dy, wzz = vz * dz, wxy = vx * dy;
    acc[14] += wxx * dx; acc[15] += wyy * dy; acc[16] += wzz * dz;
    acc[17] += wxx * dy; acc[18] += wxx * dz; acc[19] += wyy * dx;
    acc[20] += wzz * dx; acc[21] += wyy * dz; acc[22] += wzz * dy;
    acc[23] += wxy * dz;
}

// lrf_update's periodic shift L*nint((x_sw - cent)/L) of a far source group
// (switch atom sw at hi/lo sh/sl) about the target centre c (float offsets);
// recomputed from the FP64 coordinates and centre when the float quotient is
// within 1e-4 of a half-integer, where float rounding could pick the other image.
__device__ __forceinline__ float3 lrf_box_shift(const DevSys &S, const TrajInfo &T, const float4 sh, const float4 sl,
                                                float cx, float cy, float cz, int sw, int t) {
    const float u[3] = {((sh.x - cx) + sl.x) * T.iboxf[0], ((sh.y - cy) + sl.y) * T.iboxf[1],
                        ((sh.z - cz) + sl.z) * T.iboxf[2]};
    float o[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float a = fabsf(u[k]);
        float n = rintf(u[k]);
        if (fabsf(a - floorf(a) - 0.5f) < 1e-4f)
            n = (float)round((S.x[3 * sw + k] - S.g_cent[3 * t + k]) * T.ibox[k]);
        o[k] = T.boxf[k] * n;
    }
    return make_float3(o[0], o[1], o[2]);
}

// Phase 1 of the scan: one thread per target charge group, one block per
// (128 targets, source chunk of QG_TPC shared-memory tiles of the same
// trajectory).  Near groups (inside the pp/pw/ww cut-off) go to the target's
// chunk segment of near groups (a full list: both directions are found); far
// groups inside RcLRF add their non-Q atoms to the target's multipole
// expansion (lrf_update, src/md.f90:5896-5981), accumulated as 24 symmetric
// FP32 sums per chunk.
// PBC: the periodic-box form (nbpplist_box_lrf :8190, nbpwlist_box_lrf :9431,
// nbwwlist_box_lrf :11023): minimum-image switch-atom distances, and each far
// group's atoms shifted by the periodic image of its switch atom relative to
// the target centre (lrf_update :5905-5917).
template <bool ANY, bool PBC>
__global__ void __launch_bounds__(QG_BLOCK, QG_SCAN_MINB) k_scan(DevSys S, const int *blk_t0, const int *blk_tn, const int *blk_traj,
                                                   const int *blk_chunk) {
    __shared__ float4 s_hi[QG_TILE_G], s_lo[QG_TILE_G];
    __shared__ int s_meta[QG_TILE_G], s_rep[QG_TILE_G], s_aoff[QG_TILE_G + 1];
    __shared__ float4 s_atom[QG_TILE_A];
    __shared__ float s_ext[QG_TILE_G];
    const int b = blockIdx.x;
    const TrajInfo &T = S.traj[blk_traj[b]];
    const int chunk = blk_chunk[b];
    const int tid = threadIdx.x;
    const int t = blk_t0[b] + tid;
    const bool valid = tid < blk_tn[b];
    int kind_t = 0, rt = 0;
    bool active = false;
    float4 th = make_float4(0, 0, 0, 0), tl = th;
    float cx = 0, cy = 0, cz = 0;
    float ext_t = 0.f;
    int ta0 = 0, ta1 = 0;
    const bool any_atom = ANY && T.any_atom != 0;
    // any-atom test: the target's first QG_TREG atoms in registers (a water
    // target takes part by its O only); tlast = the group's last atom
    // (per-thread slots in shared memory keep them out of the registers)
    __shared__ float4 s_tp[ANY ? QG_TREG + 1 : 1][QG_BLOCK];
    __shared__ int s_ti[ANY ? QG_TREG + 1 : 1][QG_BLOCK];
    int ntreg = 0;
    if (valid) {
        kind_t = S.g_kind[t];
        rt = S.g_switch[t];
        active = !S.g_excl[t];
        th = S.pos[rt]; tl = S.poslo[rt];
        const float4 c = S.g_centf[t];
        cx = c.x; cy = c.y; cz = c.z; ext_t = c.w;
        ta0 = S.g_start[t]; ta1 = kind_t ? ta0 + 1 : S.g_start[t + 1];
        if (any_atom) {
            ntreg = min(ta1 - ta0, QG_TREG);
            for (int k = 0; k < ntreg; ++k) {
                const int a = S.g_atoms[ta0 + k];
                s_ti[k][tid] = a; s_tp[k][tid] = S.pos[a];
            }
            const int la = kind_t ? rt : S.g_atoms[S.g_start[t + 1] - 1];
            s_ti[ANY ? QG_TREG : 0][tid] = la; s_tp[ANY ? QG_TREG : 0][tid] = S.pos[la];
        }
    }
    const long long slot = T.scr0 + (long long)chunk * T.ncgp + (t - T.grp0);
    int *nbseg = S.scr_nb + (size_t)slot * QG_CAPC;
    int2 *shseg = (ANY && PBC && S.scr_sha) ? S.scr_sha + (size_t)slot * QG_CAPC : nullptr;
    float acc[QG_NLRF];
#pragma unroll
    for (int k = 0; k < QG_NLRF; ++k) acc[k] = 0.f;
    int cntw = 0, cnts = 0;
    const float rc2_lrf = T.rc2_lrf;
    const bool lrf = T.use_lrf != 0;
    const int it0 = chunk * QG_TPC, it1 = min(T.ntile, it0 + QG_TPC);
    for (int it = it0; it < it1; ++it) {
        const int tile = T.tile0 + it;
        const int g0 = S.tile_g0[tile], g1 = S.tile_g1[tile], ng = g1 - g0;
        const int ab = S.g_start[g0], ae = S.g_start[g1];
        __syncthreads();
        for (int k = tid; k < ng; k += blockDim.x) {
            int g = g0 + k, ra = S.g_switch[g];
            s_hi[k] = S.pos[ra]; s_lo[k] = S.poslo[ra];
            s_ext[k] = S.g_centf[g].w;
            s_meta[k] = S.g_kind[g] | (S.g_excl[g] ? 2 : 0);
            s_rep[k] = ra;
            s_aoff[k] = S.g_start[g] - ab;
            if (k == ng - 1) s_aoff[ng] = ae - ab;
        }
        for (int k = tid; k < ae - ab; k += blockDim.x) {
            int a = S.g_atoms[ab + k];
            float4 p = S.pos[a];
            if (S.aq[a] >= 0) p.w = 0.f;   // Q atoms do not contribute to the LRF
            s_atom[k] = p;
        }
        __syncthreads();
        if (active) {
            for (int s = 0; s < ng; ++s) {
                const int g = g0 + s;
                const int meta = s_meta[s];
                if ((meta & 2) || g == t) continue;
                const int kind_s = meta & 1;
                float rc2; double drc2;
                if (kind_t & kind_s) { rc2 = T.rc2_ww; drc2 = T.drc2_ww; }
                else if (kind_t | kind_s) { rc2 = T.rc2_pw; drc2 = T.drc2_pw; }
                else { rc2 = T.rc2_pp; drc2 = T.drc2_pp; }
                float3 d = dpos(th, tl, s_hi[s], s_lo[s]);
                if (PBC) d = f3sub(d, box_shift(T, d));
                float d2 = d.x * d.x + d.y * d.y + d.z * d.z;
                bool near_, far_lrf;
                int2 rec = make_int2(-1, -1);
                if (ANY && PBC && any_atom && T.pbc && !(kind_t & kind_s)) {
                    // nbpplis2_box_lrf (src/md.f90:7241-7439) / nbpwlis2_box_lrf
                    // (:8745-8900): minimum-image atom pairs (a water counts by
                    // its O) in the reference's loop order -- the outer group is
                    // the solute group of a solute-water pair, and of a solute
                    // pair the group the count-once rule keeps first.  The first
                    // pair inside the cut-off is the pair's shift record; not
                    // inside, the LRF holds when some pair lies within RcLRF.
                    const int sa0 = ab + s_aoff[s], sa1 = ab + s_aoff[s + 1];
                    const int sb1 = kind_s ? sa0 + 1 : sa1;
                    const float ea = kind_t ? 0.f : ext_t, eb = kind_s ? 0.f : s_ext[s];
                    const float rn = sqrtf(rc2) + ea + eb, rf = sqrtf(rc2_lrf) + ea + eb;
                    near_ = false;
                    far_lrf = false;
                    if (d2 <= rf * rf * (1.f + 1e-4f)) {
                        const int tl = t - T.grp0, sl = g - T.grp0;
                        const bool t_outer = kind_t != kind_s
                                                 ? kind_t == 0
                                                 : !((tl > sl && ((tl + sl) & 1) == 0) || (tl < sl && ((tl + sl) & 1) == 1));
                        const bool test_near = d2 <= rn * rn * (1.f + 1e-4f);
                        bool anyl = false;
                        const int nt = ta1 - ta0, nsrc = sb1 - sa0;
                        const int no = t_outer ? nt : nsrc, ni = t_outer ? nsrc : nt;
                        for (int io = 0; io < no && !near_; ++io)
                            for (int ii = 0; ii < ni && !near_; ++ii) {
                                const int kt = t_outer ? io : ii, ks = t_outer ? ii : io;
                                const int ia = kt < ntreg ? s_ti[kt][tid] : S.g_atoms[ta0 + kt];
                                const float4 pa = kt < ntreg ? s_tp[kt][tid] : S.pos[ia];
                                const int jb = S.g_atoms[sa0 + ks];
                                const float r2 = d2hi_box(pa, s_atom[sa0 + ks - ab], T);
                                if (test_near && within_hi_box(r2, rc2, drc2, S.x, ia, jb, T)) {
                                    near_ = true;
                                    rec = make_int2(ia, jb);
                                } else if (lrf && !anyl) {
                                    anyl = within_hi_box(r2, rc2_lrf, T.drc2_lrf, S.x, ia, jb, T);
                                }
                            }
                        far_lrf = !near_ && anyl;
                    }
                } else if (any_atom && !(kind_t & kind_s)) {
                    // nbpplis2_lrf (src/md.f90:7518-7545) / nbpwlis2_lrf
                    // (:8970-8985): inside when any atom pair is within the
                    // cut-off (a water counts by its O); else the LRF test
                    // on the last atom pair the reference's loop computed
                    const int sa0 = ab + s_aoff[s], sa1 = ab + s_aoff[s + 1];
                    const int sb1 = kind_s ? sa0 + 1 : sa1;   // a water source: its O only
                    near_ = false;
                    const float reach = sqrtf(rc2) + (kind_t ? 0.f : ext_t) + (kind_s ? 0.f : s_ext[s]);
                    if (d2 <= reach * reach * (1.f + 1e-4f)) {
                        for (int kb = sa0; kb < sb1 && !near_; ++kb) {
                            const float4 pb = s_atom[kb - ab];
                            const int jb = S.g_atoms[kb];
                            for (int k = 0; k < ntreg && !near_; ++k)
                                near_ = within_hi(d2hi(s_tp[k][tid], pb), rc2, drc2, S.x, s_ti[k][tid], jb);
                            for (int ka = ta0 + QG_TREG; ka < ta1 && !near_; ++ka) {
                                const int ia = S.g_atoms[ka];
                                near_ = within_hi(d2hi(S.pos[ia], pb), rc2, drc2, S.x, ia, jb);
                            }
                        }
                    }
                    far_lrf = false;
                    if (!near_ && lrf) {
                        const int lk = kind_s ? sa0 : sa1 - 1;
                        const int lt = ANY ? QG_TREG : 0;
                        far_lrf = within_hi(d2hi(s_tp[lt][tid], s_atom[lk - ab]), rc2_lrf, T.drc2_lrf, S.x,
                                            s_ti[lt][tid], S.g_atoms[lk]);
                    }
                } else if (PBC) {
                    near_ = within_box(d2, rc2, drc2, S.x, rt, s_rep[s], T);
                    far_lrf = !near_ && lrf && within_box(d2, rc2_lrf, T.drc2_lrf, S.x, rt, s_rep[s], T);
                } else {
                    near_ = within(d2, rc2, drc2, S.x, rt, s_rep[s]);
                    far_lrf = !near_ && lrf && within(d2, rc2_lrf, T.drc2_lrf, S.x, rt, s_rep[s]);
                }
                if (near_) {
                    // at most QG_CAPC groups per chunk: water neighbours (as
                    // their O atom) from the front, solute groups from the back
                    if (kind_s) {
                        if (shseg) shseg[cntw] = rec;
                        nbseg[cntw++] = s_rep[s];
                    } else {
                        if (shseg) shseg[QG_CAPC - 1 - cnts] = rec;
                        nbseg[QG_CAPC - 1 - cnts++] = g;
                    }
                } else if (far_lrf) {
                    const int k0 = s_aoff[s];
                    // in a box the expansion centre moves by the periodic
                    // image of the source's switch atom (lrf_update :5905-5917)
                    float ex = cx, ey = cy, ez = cz;
                    if (PBC) {
                        const float3 sh = lrf_box_shift(S, T, s_hi[s], s_lo[s], cx, cy, cz, s_rep[s], t);
                        ex = cx + sh.x; ey = cy + sh.y; ez = cz + sh.z;
                    }
                    if (kind_s) {
                        // a water: its three (charged) atoms unrolled, so their
                        // independent rsqrt chains overlap; same order of sums
                        const float4 p0 = s_atom[k0], p1 = s_atom[k0 + 1], p2 = s_atom[k0 + 2];
                        lrf_acc(acc, p0, ex, ey, ez);
                        lrf_acc(acc, p1, ex, ey, ez);
                        lrf_acc(acc, p2, ex, ey, ez);
                    } else {
                        for (int k = k0; k < s_aoff[s + 1]; ++k) {
                            const float4 p = s_atom[k];
                            if (p.w == 0.f) continue;
                            lrf_acc(acc, p, ex, ey, ez);
                        }
                    }
                }
            }
        }
    }
    if (!valid) return;
    S.scr_cnt[slot] = cntw | (cnts << 16);
    float *ph = S.scr_phi + (size_t)slot * QG_NLRF;
#pragma unroll
    for (int k = 0; k < QG_NLRF; ++k) ph[k] = acc[k];
}

// Phase 2: one warp per target group folds the chunks in order -- lane k
// sums LRF component k (FP32; at most a few tens of chunk partials), the
// lanes copy the chunks' near-group segments into the neighbour list (water
// entries of every chunk first, then solute entries) -- and lane 0 forms the
// symmetric Taylor coefficients.  No FP64: this runs over every group.
template <bool SHA>
__global__ void k_scan_reduce(DevSys S, int gb, int gn) {
    const int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (k >= gn) return;
    const int t = gb + k;
    const TrajInfo &T = S.traj[S.g_traj[t]];
    const bool ex = S.g_excl[t];
    const int cap = S.nb_cap;
    int *lst = S.nb_list + (size_t)t * cap;
    const int nch = T.nchunk;
    const size_t base = (size_t)(T.scr0 + (t - T.grp0)), stride = (size_t)T.ncgp;   // slot(c) = base + c*stride
    // LRF partials in chunk order, eight chunks' loads in flight at a time
    float acc = 0.f;
    if (lane < QG_NLRF) {
        int c = 0;
        for (; c + 8 <= nch; c += 8) {
            float v[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) v[u] = S.scr_phi[(base + (size_t)(c + u) * stride) * QG_NLRF + lane];
#pragma unroll
            for (int u = 0; u < 8; ++u) acc += v[u];
        }
        for (; c < nch; ++c) acc += S.scr_phi[(base + (size_t)c * stride) * QG_NLRF + lane];
    }
    // near groups: every chunk's counts (chunk r*32 + lane in round r), their
    // offsets in chunk order by warp prefix sums -- water entries of all
    // chunks first, then solute entries -- and the segments copied four
    // chunks at a time (their loads in flight together)
    int cnt = 0, nwat = 0;
    if (!ex) {
        int wtot = 0, stot = 0;
        for (int r0 = 0; r0 < nch; r0 += 32) {
            const int c = r0 + lane;
            const int cc = c < nch ? S.scr_cnt[base + (size_t)c * stride] : 0;
            wtot += __reduce_add_sync(0xffffffffu, cc & 0xffff);
            stot += __reduce_add_sync(0xffffffffu, cc >> 16);
        }
        nwat = wtot;
        cnt = wtot + stot;
        int ow = 0, os = wtot;   // running offsets before the current round
        for (int r0 = 0; r0 < nch; r0 += 32) {
            const int c = r0 + lane;
            const int cc = c < nch ? S.scr_cnt[base + (size_t)c * stride] : 0;
            const int nw = cc & 0xffff, ns = cc >> 16;
            int pw = nw, ps = ns;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int yw = __shfl_up_sync(0xffffffffu, pw, o), ys = __shfl_up_sync(0xffffffffu, ps, o);
                if (lane >= o) { pw += yw; ps += ys; }
            }
            const int offw = ow + pw - nw, offs = os + ps - ns;
            const int nr = min(32, nch - r0);
            for (int j0 = 0; j0 < nr; j0 += 4) {
                int vw[4][QG_CAPC / 32], vs[4][QG_CAPC / 32], dw[4], ds[4], kw[4], ks[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int j = min(j0 + u, 31);
                    const bool on = j0 + u < nr;
                    kw[u] = on ? __shfl_sync(0xffffffffu, nw, j) : 0;
                    ks[u] = on ? __shfl_sync(0xffffffffu, ns, j) : 0;
                    dw[u] = __shfl_sync(0xffffffffu, offw, j);
                    ds[u] = __shfl_sync(0xffffffffu, offs, j);
                    const int *seg = S.scr_nb + (base + (size_t)(r0 + j) * stride) * QG_CAPC;
#pragma unroll
                    for (int h = 0; h < QG_CAPC / 32; ++h) {
                        const int k = lane + 32 * h;
                        vw[u][h] = k < kw[u] ? seg[k] : 0;
                        vs[u][h] = k < ks[u] ? seg[QG_CAPC - 1 - k] : 0;
                    }
                }
#pragma unroll
                for (int u = 0; u < 4; ++u)
#pragma unroll
                    for (int h = 0; h < QG_CAPC / 32; ++h) {
                        const int k = lane + 32 * h;
                        if (k < kw[u] && dw[u] + k < cap) lst[dw[u] + k] = vw[u][h];
                        if (k < ks[u] && ds[u] + k < cap) lst[ds[u] + k] = vs[u][h];
                    }
                // any-atom lists in a box: the shift records go along
                if (SHA) {
                    int2 *rl = S.nb_sha + (size_t)t * cap;
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const int2 *sseg = S.scr_sha + (base + (size_t)(r0 + min(j0 + u, 31)) * stride) * QG_CAPC;
                        for (int k = lane; k < kw[u]; k += 32)
                            if (dw[u] + k < cap) rl[dw[u] + k] = sseg[k];
                        for (int k = lane; k < ks[u]; k += 32)
                            if (ds[u] + k < cap) rl[ds[u] + k] = sseg[QG_CAPC - 1 - k];
                    }
                }
            }
            ow += __shfl_sync(0xffffffffu, pw, 31);
            os += __shfl_sync(0xffffffffu, ps, 31);
        }
    }
    float a[QG_NLRF];
#pragma unroll
    for (int k = 0; k < QG_NLRF; ++k) a[k] = __shfl_sync(0xffffffffu, acc, k);
    if (lane < QG_NLRF) S.g_phi[(size_t)t * QG_NLRF + lane] = acc;
    if (lane != 0) return;
    S.nb_nw[t] = nwat < cap ? nwat : cap;
    S.nb_count[t] = cnt < cap ? cnt : cap;
    if (cnt > cap) atomicOr(S.status, ST_LIST_OVERFLOW);
    float *pf = S.g_phif + (size_t)t * QG_NPHI;
    const float q1x = a[5], q1y = a[6], q1z = a[7];
    pf[0] = a[0];
    pf[1] = -a[2]; pf[2] = -a[3]; pf[3] = -a[4];
    pf[4] = a[8] - a[1]; pf[5] = a[9] - a[1]; pf[6] = a[10] - a[1];
    pf[7] = a[11]; pf[8] = a[12]; pf[9] = a[13];
    pf[10] = 5.f * a[14] + 3.f * q1x;
    pf[11] = 5.f * a[15] + 3.f * q1y;
    pf[12] = 5.f * a[16] + 3.f * q1z;
    pf[13] = 5.f * a[17] + q1y;   // xxy
    pf[14] = 5.f * a[18] + q1z;   // xxz
    pf[15] = 5.f * a[19] + q1x;   // xyy
    pf[16] = 5.f * a[20] + q1x;   // xzz
    pf[17] = 5.f * a[21] + q1z;   // yyz
    pf[18] = 5.f * a[22] + q1y;   // yzz
    pf[19] = 5.f * a[23];         // xyz
}

// Q-atom list membership (nbqplist src/md.f90:10215-10322, nbqwlist
// :10464-10549): waters whose O and solute groups whose switch atom lie within
// Rcq of the solute centre.  Built once when Rcq > rexcl_o, as the reference.
__global__ void k_qmember(DevSys S, int first, int gb, int gn) {
    const int kk = blockIdx.x * blockDim.x + threadIdx.x;
    if (kk >= gn) return;
    const int g = gb + kk;
    const TrajInfo &T = S.traj[S.g_traj[g]];
    if (!first && T.q_static) return;
    if (T.nqat == 0) return;
    int sw = S.g_switch[g];
    if (T.pbc) {
        // nbqwlist_box :10554 / nbqplist_box :10327: within Rcq of the Q
        // switching atom (minimum image); a solute group by any of its atoms,
        // the first such atom fixing the group's periodic shift
        const int q = T.qswitch;
        int in_at = -1;
        if (S.g_kind[g]) {
            if (dist2_exact_box(S.x, sw, q, T) <= T.drcq2) in_at = sw;
            S.qw_member[sw] = in_at >= 0 ? 1 : 0;
        } else {
            for (int k = S.g_start[g]; k < S.g_start[g + 1] && in_at < 0; ++k)
                if (dist2_exact_box(S.x, S.g_atoms[k], q, T) <= T.drcq2) in_at = S.g_atoms[k];
            S.g_qin[g] = in_at;
            for (int k = S.g_start[g]; k < S.g_start[g + 1]; ++k) {
                const int at = S.g_atoms[k];
                S.qp_member[at] = (in_at >= 0 && !S.qp_skip[at]) ? 1 : 0;
            }
        }
        return;
    }
    double a = S.x[3 * sw] - T.xpcent[0], b = S.x[3 * sw + 1] - T.xpcent[1], c = S.x[3 * sw + 2] - T.xpcent[2];
    bool in = !S.g_excl[g] && (a * a + b * b + c * c <= T.drcq2);
    if (T.any_atom && !S.g_kind[g] && !S.g_excl[g]) {
        // nbqplis2, src/md.f90:9946-10071: any atom of the group within Rcq
        in = false;
        for (int k = S.g_start[g]; k < S.g_start[g + 1] && !in; ++k) {
            const int at = S.g_atoms[k];
            a = S.x[3 * at] - T.xpcent[0]; b = S.x[3 * at + 1] - T.xpcent[1]; c = S.x[3 * at + 2] - T.xpcent[2];
            in = a * a + b * b + c * c <= T.drcq2;
        }
    }
    if (S.g_kind[g]) {
        S.qw_member[sw] = in ? 1 : 0;
    } else {
        for (int k = S.g_start[g]; k < S.g_start[g + 1]; ++k) {
            int at = S.g_atoms[k];
            S.qp_member[at] = (in && !S.qp_skip[at]) ? 1 : 0;
        }
    }
}

// put_back_in_box, src/md.f90:18740-18857: one block per box trajectory.  The
// box centre follows the mean solute position (all atoms without solute)
// unless rigid_box_centre; every selected molecule whose mass centre lies
// outside the box moves by one box length per axis, in FP64 on x, and its
// float coordinates (and water record) are re-formed.
__global__ void k_put_back(DevSys S, const int *pb_traj) {
    const int traj = pb_traj[blockIdx.x];
    const TrajInfo &T = S.traj[traj];
    __shared__ double red[3][256];
    __shared__ double bc[3];
    const int tid = threadIdx.x;
    if (!T.rigid_box) {
        const int n = T.nat_solute > 0 ? T.nat_solute : T.natom;
        double c[3] = {0.0, 0.0, 0.0};
        for (int i = tid; i < n; i += blockDim.x)
#pragma unroll
            for (int a = 0; a < 3; ++a) c[a] += S.x[3 * (T.atom0 + i) + a];
#pragma unroll
        for (int a = 0; a < 3; ++a) red[a][tid] = c[a];
        __syncthreads();
        for (int w = blockDim.x / 2; w > 0; w >>= 1) {
            if (tid < w)
#pragma unroll
                for (int a = 0; a < 3; ++a) red[a][tid] += red[a][tid + w];
            __syncthreads();
        }
        if (tid < 3) S.boxc[3 * traj + tid] = red[tid][0] / n;
        __syncthreads();
    }
    if (tid < 3) bc[tid] = S.boxc[3 * traj + tid];
    __syncthreads();
    const int m0 = T.put_solute ? 0 : T.nsolute_mol, m1 = T.put_solvent ? T.nmol : T.nsolute_mol;
    for (int m = m0 + tid; m < m1; m += blockDim.x) {
        const int a0 = S.mol_start[T.mol0 + m], a1 = S.mol_start[T.mol0 + m + 1];
        double cm[3] = {0.0, 0.0, 0.0}, mt = 0.0;
        for (int j = a0; j < a1; ++j) mt += S.mass[j];
        for (int j = a0; j < a1; ++j)
#pragma unroll
            for (int a = 0; a < 3; ++a) cm[a] = __dadd_rn(cm[a], __dmul_rn(S.x[3 * j + a], S.mass[j]));
        bool moved = false;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const double c = __dmul_rn(cm[a], 1.0 / mt);
            const double hi = bc[a] + T.box[a] / 2, lo = bc[a] - T.box[a] / 2;
            const double mv = c > hi ? -T.box[a] : (c < lo ? T.box[a] : 0.0);
            if (mv != 0.0) {
                moved = true;
                for (int j = a0; j < a1; ++j) S.x[3 * j + a] = S.x[3 * j + a] + mv;
            }
        }
        if (!moved) continue;
        for (int j = a0; j < a1; ++j) {
            const double r0 = S.x[3 * j] - T.origin[0], r1 = S.x[3 * j + 1] - T.origin[1], r2 = S.x[3 * j + 2] - T.origin[2];
            float4 h, l;
            h.x = (float)r0; h.y = (float)r1; h.z = (float)r2; h.w = S.pos[j].w;
            l.x = (float)(r0 - (double)h.x); l.y = (float)(r1 - (double)h.y); l.z = (float)(r2 - (double)h.z); l.w = 0.f;
            S.pos[j] = h;
            S.poslo[j] = l;
        }
        if (a1 - a0 == 3 && a0 >= T.atom0 + T.nat_solute) {
            float4 h[3], l[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) { h[k] = S.pos[a0 + k]; l[k] = S.poslo[a0 + k]; }
            put_wrec(S.wrec + a0, h, l);
        }
    }
}

static inline int nblk(int n, int b) { return (n + b - 1) / b; }

void launch_put_back(const DevSys &S, const BlockTables &B, LaunchCtx &L) {
    if (!B.npb) return;
    prof_begin(L, "k_put_back");
    k_put_back<<<B.npb, 256, 0, L.stream>>>(S, B.pb_traj);
    prof_end(L);
    (*L.nlaunch)++;
}

void launch_wrec(const DevSys &S, const BlockTables &B, LaunchCtx &L) {
    if (!B.nwgrp) return;
    prof_begin(L, "k_wrec");
    k_wrec<<<nblk(B.nwgrp, 256), 256, 0, L.stream>>>(S, B.wgrp, B.nwgrp);
    prof_end(L);
    (*L.nlaunch)++;
}
void launch_mirror_range(const DevSys &S, LaunchCtx &L, int a0, int n) {
    if (n <= 0) return;
    prof_begin(L, "k_mirror_range");
    k_mirror_range<<<nblk(n, 256), 256, 0, L.stream>>>(S, a0, n);
    prof_end(L);
    (*L.nlaunch)++;
}
void launch_mirror(const DevSys &S, const BlockTables &B, LaunchCtx &L) {
    prof_begin(L, "k_mirror");
    k_mirror<<<nblk(S.natom, 256), 256, 0, L.stream>>>(S);
    prof_end(L);
    (*L.nlaunch)++;
    launch_wrec(S, B, L);
}
void launch_centers(const DevSys &S, const BlockTables &B, LaunchCtx &L) {
    prof_begin(L, "k_centers");
    k_centers<<<nblk(B.ng, 256), 256, 0, L.stream>>>(S, B.g0, B.ng);
    prof_end(L);
    (*L.nlaunch)++;
}
void launch_scan(const DevSys &S, const BlockTables &B, LaunchCtx &L) {
    prof_begin(L, "k_scan");
    // one form covers the whole batch: both flags per trajectory when the
    // batch holds any-atom lists and periodic boxes
    if (B.any_atom && B.pbc)
        k_scan<true, true><<<B.nscan, QG_BLOCK, 0, L.stream>>>(S, B.scan_t0, B.scan_tn, B.scan_traj, B.scan_chunk);
    else if (B.any_atom)
        k_scan<true, false><<<B.nscan, QG_BLOCK, 0, L.stream>>>(S, B.scan_t0, B.scan_tn, B.scan_traj, B.scan_chunk);
    else if (B.pbc)
        k_scan<false, true><<<B.nscan, QG_BLOCK, 0, L.stream>>>(S, B.scan_t0, B.scan_tn, B.scan_traj, B.scan_chunk);
    else
        k_scan<false, false><<<B.nscan, QG_BLOCK, 0, L.stream>>>(S, B.scan_t0, B.scan_tn, B.scan_traj, B.scan_chunk);
    prof_end(L);
    (*L.nlaunch)++;
    prof_begin(L, "k_scan_reduce");
    if (S.nb_sha) k_scan_reduce<true><<<nblk(B.ng * 32, 128), 128, 0, L.stream>>>(S, B.g0, B.ng);
    else k_scan_reduce<false><<<nblk(B.ng * 32, 128), 128, 0, L.stream>>>(S, B.g0, B.ng);
    prof_end(L);
    (*L.nlaunch)++;
}
void launch_qmember(const DevSys &S, const BlockTables &B, LaunchCtx &L, int first) {
    prof_begin(L, "k_qmember");
    k_qmember<<<nblk(B.ng, 256), 256, 0, L.stream>>>(S, first, B.g0, B.ng);
    prof_end(L);
    (*L.nlaunch)++;
}
