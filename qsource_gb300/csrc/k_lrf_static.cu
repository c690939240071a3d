// k_lrf_static.cu -- qgpu_lrf_scan_static: the charge-group scan (near-group
// counts and LRF multipoles of the groups beyond the cut-off) for one system
// whose arrays the caller already holds on the device, with its chunk
// partials kept in a fixed device array of this file instead of memory the
// engine allocates.  Meant for callers that must not allocate device memory:
// code whose device memory is owned by a framework's own allocator or a pool
// sized once at start-up, and loops where a cudaMalloc (which may synchronise
// the whole device) is not allowed in the middle of a time step.
//
// The arithmetic is that of k_scan / k_scan_reduce (k_lists.cu): the same
// hi/lo float coordinates relative to `origin`, the same FP32 prefilter with
// the exact FP64 recheck of the cut-off, FP32 multipole sums per source chunk
// folded in FP64.  Only the split of the source groups into chunks differs,
// so the multipoles agree with qgpu_build_lists + qgpu_get_lrf to FP32
// rounding and the near-group counts agree exactly.
#include <mutex>

#include "qgpu_internal.cuh"

#define QS_SLOTS 65536            // (chunk, group) partial slots
#define QS_SLOT_FLOATS 32         // 24 LRF sums + near count + padding (128 B)
#define QS_CHUNK_MIN 256          // source groups per chunk at the least

// The scratch: QS_SLOTS slots of 128 bytes (8 MiB), held by every device that
// loads the library until the process exits.  Each slot is written in full by
// phase 1 before phase 2 reads it, so no call has to clear it.
static __device__ __align__(256) float qs_scratch[QS_SLOTS * QS_SLOT_FLOATS];

struct QsArgs {
    int ngroup, nchunk, chunk_groups;
    const double *x, *crg;
    const int *g_start, *g_atoms, *g_switch, *g_flags;
    double origin[3];
    float rc2_pp, rc2_pw, rc2_ww, rc2_lrf;
    double drc2_pp, drc2_pw, drc2_ww, drc2_lrf;
    double *lrf43;
    int *near_count;
};

// hi/lo split of x - origin, as k_mirror.
__device__ __forceinline__ void qs_hilo(const QsArgs &A, int a, float4 &h, float4 &l) {
    const double r0 = A.x[3 * a] - A.origin[0], r1 = A.x[3 * a + 1] - A.origin[1], r2 = A.x[3 * a + 2] - A.origin[2];
    h.x = (float)r0; h.y = (float)r1; h.z = (float)r2; h.w = (float)A.crg[a];
    l.x = (float)(r0 - (double)h.x); l.y = (float)(r1 - (double)h.y); l.z = (float)(r2 - (double)h.z); l.w = 0.f;
}

// group centre, as k_centers (FP64 mean of the members in list order)
__device__ __forceinline__ void qs_center(const QsArgs &A, int g, double c[3]) {
    double c0 = 0, c1 = 0, c2 = 0;
    const int a0 = A.g_start[g], a1 = A.g_start[g + 1];
    for (int k = a0; k < a1; ++k) {
        const int a = A.g_atoms[k];
        c0 += A.x[3 * a]; c1 += A.x[3 * a + 1]; c2 += A.x[3 * a + 2];
    }
    const double n = (double)(a1 - a0);
    c[0] = c0 / n; c[1] = c1 / n; c[2] = c2 / n;
}

__device__ __forceinline__ bool qs_within(float d2, float rc2, double drc2, const double *x, int a, int b) {
    if (d2 < rc2 * (1.f - 1e-5f)) return true;
    if (d2 > rc2 * (1.f + 1e-5f)) return false;
    return dist2_exact(x, a, b) <= drc2;
}

// Phase 1: block (128 targets, source chunk).  Source groups of the chunk are
// staged in shared-memory tiles of at most QG_TILE_G groups and QG_TILE_A
// atoms; a single group with more atoms than a tile holds is read from
// global memory.
__global__ void __launch_bounds__(QG_BLOCK) k_scan_static(QsArgs A, float *scratch) {
    __shared__ float4 s_hi[QG_TILE_G], s_lo[QG_TILE_G];
    __shared__ int s_meta[QG_TILE_G], s_rep[QG_TILE_G], s_aoff[QG_TILE_G + 1];
    __shared__ float4 s_atom[QG_TILE_A];
    __shared__ int s_tile_end, s_big;
    const int tid = threadIdx.x;
    const int t = blockIdx.x * QG_BLOCK + tid;
    const int chunk = blockIdx.y;
    const bool valid = t < A.ngroup;
    int kind_t = 0, rt = 0;
    bool active = false;
    float4 th = make_float4(0, 0, 0, 0), tl = th;
    float cx = 0, cy = 0, cz = 0;
    if (valid) {
        kind_t = A.g_flags[t] & 1;
        active = !(A.g_flags[t] & 2);
        rt = A.g_switch[t];
        qs_hilo(A, rt, th, tl);
        double c[3];
        qs_center(A, t, c);
        cx = (float)(c[0] - A.origin[0]); cy = (float)(c[1] - A.origin[1]); cz = (float)(c[2] - A.origin[2]);
    }
    float acc[QG_NLRF];
#pragma unroll
    for (int k = 0; k < QG_NLRF; ++k) acc[k] = 0.f;
    int cnt = 0;
    const int c0 = chunk * A.chunk_groups, c1 = min(A.ngroup, c0 + A.chunk_groups);
    for (int g0 = c0; g0 < c1;) {
        __syncthreads();
        if (tid == 0) {
            // greedy tile: up to QG_TILE_G groups and QG_TILE_A atoms
            int g = g0, na = 0;
            while (g < c1 && g - g0 < QG_TILE_G) {
                const int n = A.g_start[g + 1] - A.g_start[g];
                if (na + n > QG_TILE_A) break;
                na += n; ++g;
            }
            s_big = (g == g0);          // first group alone exceeds a tile
            s_tile_end = s_big ? g0 + 1 : g;
        }
        __syncthreads();
        const int g1 = s_tile_end, ng = g1 - g0;
        const bool big = s_big != 0;
        const int ab = A.g_start[g0], ae = A.g_start[g1];
        for (int k = tid; k < ng; k += blockDim.x) {
            const int g = g0 + k, ra = A.g_switch[g];
            float4 h, l;
            qs_hilo(A, ra, h, l);
            s_hi[k] = h; s_lo[k] = l;
            s_meta[k] = A.g_flags[g] & 3;
            s_rep[k] = ra;
            s_aoff[k] = A.g_start[g] - ab;
            if (k == ng - 1) s_aoff[ng] = ae - ab;
        }
        if (!big)
            for (int k = tid; k < ae - ab; k += blockDim.x) {
                float4 h, l;
                qs_hilo(A, A.g_atoms[ab + k], h, l);
                s_atom[k] = h;
            }
        __syncthreads();
        if (active) {
            for (int s = 0; s < ng; ++s) {
                const int g = g0 + s;
                const int meta = s_meta[s];
                if ((meta & 2) || g == t) continue;
                const int kind_s = meta & 1;
                float rc2; double drc2;
                if (kind_t & kind_s) { rc2 = A.rc2_ww; drc2 = A.drc2_ww; }
                else if (kind_t | kind_s) { rc2 = A.rc2_pw; drc2 = A.drc2_pw; }
                else { rc2 = A.rc2_pp; drc2 = A.drc2_pp; }
                const float3 d = dpos(th, tl, s_hi[s], s_lo[s]);
                const float d2 = d.x * d.x + d.y * d.y + d.z * d.z;
                if (qs_within(d2, rc2, drc2, A.x, rt, s_rep[s])) {
                    ++cnt;
                } else if (qs_within(d2, A.rc2_lrf, A.drc2_lrf, A.x, rt, s_rep[s])) {
                    for (int k = s_aoff[s]; k < s_aoff[s + 1]; ++k) {
                        float4 p;
                        if (big) { float4 l; qs_hilo(A, A.g_atoms[ab + k], p, l); }
                        else p = s_atom[k];
                        if (p.w == 0.f) continue;
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
                }
            }
        }
        g0 = g1;
    }
    if (!valid) return;
    float *slot = scratch + ((size_t)chunk * A.ngroup + t) * QS_SLOT_FLOATS;
#pragma unroll
    for (int k = 0; k < QG_NLRF; ++k) slot[k] = acc[k];
    slot[QG_NLRF] = __int_as_float(cnt);
}

// index of the symmetric third-moment sum for components (i, j, k)
__device__ __forceinline__ int qs_p3(int i, int j, int k) {
    int a = min(i, min(j, k)), c = max(i, max(j, k)), b = i + j + k - a - c;
    if (a == c) return 14 + a;                          // xxx yyy zzz
    if (a == 0 && b == 0) return c == 1 ? 17 : 18;      // xxy xxz
    if (a == 0 && b == 1 && c == 1) return 19;          // xyy
    if (a == 0 && b == 2) return 20;                    // xzz
    if (a == 1 && b == 1) return 21;                    // yyz
    if (a == 1 && b == 2) return 22;                    // yzz
    return 23;                                          // xyz
}

// Phase 2: one warp per group folds the chunk partials in chunk order (lane k
// sums component k in FP64) and writes the 43-double LRF record (centre,
// phi0, phi1, phi2, phi3 of LRF_TYPE, src/md.f90:444-450) and the count.
__global__ void k_scan_static_reduce(QsArgs A, const float *scratch) {
    const int t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (t >= A.ngroup) return;
    double acc = 0.0;
    int cnt = 0;
    for (int c = 0; c < A.nchunk; ++c) {
        const float *slot = scratch + ((size_t)c * A.ngroup + t) * QS_SLOT_FLOATS;
        if (lane < QG_NLRF) acc += (double)slot[lane];
        cnt += __float_as_int(slot[QG_NLRF]);
    }
    double a[QG_NLRF];
#pragma unroll
    for (int k = 0; k < QG_NLRF; ++k) a[k] = __shfl_sync(0xffffffffu, acc, k);
    double *o = A.lrf43 + 43 * (size_t)t;
    if (lane == 0) {
        double c[3];
        qs_center(A, t, c);
        o[0] = c[0]; o[1] = c[1]; o[2] = c[2];
        o[3] = a[0];
        o[4] = -a[2]; o[5] = -a[3]; o[6] = -a[4];
        A.near_count[t] = cnt;
    }
    // phi2 (9 entries) on lanes 0..8, phi3 (27 entries) on lanes 0..26
    if (lane < 9) {
        const int i = lane / 3, j = lane % 3;
        const int p2[3][3] = {{8, 11, 12}, {11, 9, 13}, {12, 13, 10}};
        o[7 + lane] = a[p2[i][j]] - (i == j ? a[1] : 0.0);
    }
    if (lane < 27) {
        const int i = lane / 9, j = (lane / 3) % 3, k = lane % 3;
        double val = 5.0 * a[qs_p3(i, j, k)];
        if (i == j) val += a[5 + k];
        if (i == k) val += a[5 + j];
        if (j == k) val += a[5 + i];
        o[16 + lane] = val;
    }
}

// Device address of qs_scratch for each device, resolved by the first call on
// that device (with it current).
static std::mutex qs_mutex;
static float *qs_addr[64];

static int qs_scratch_on_current_device(float **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return qgpu_fail(QGPU_E_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
    if (dev < 0 || dev >= 64) return qgpu_fail(QGPU_E_UNSUPPORTED, "device ordinal %d beyond 63", dev);
    std::lock_guard<std::mutex> lock(qs_mutex);
    if (!qs_addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, qs_scratch);
        if (e != cudaSuccess || !p)
            return qgpu_fail(QGPU_E_CUDA, "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
        qs_addr[dev] = (float *)p;
    }
    *out = qs_addr[dev];
    return 0;
}

extern "C" int qgpu_lrf_scan_static(int32_t ngroup, const double *x, const double *crg, const int32_t *g_start,
                                    const int32_t *g_atoms, const int32_t *g_switch, const int32_t *g_flags,
                                    const double *origin, double rc_pp, double rc_pw, double rc_ww, double rc_lrf,
                                    double *lrf43, int32_t *near_count, void *stream) {
    if (ngroup < 0 || !x || !crg || !g_start || !g_atoms || !g_switch || !g_flags || !origin || !lrf43 ||
        !near_count)
        return qgpu_fail(QGPU_E_INVALID, "qgpu_lrf_scan_static: bad arguments");
    if (ngroup > QS_SLOTS)
        return qgpu_fail(QGPU_E_INVALID, "qgpu_lrf_scan_static: %d charge groups exceed the static scratch limit of %d",
                         ngroup, QS_SLOTS);
    if (!(rc_pp > 0 && rc_pw > 0 && rc_ww > 0 && rc_lrf > 0))
        return qgpu_fail(QGPU_E_INVALID, "qgpu_lrf_scan_static: cut-offs must be positive");
    if (ngroup == 0) return 0;
    float *scratch = nullptr;
    int rc = qs_scratch_on_current_device(&scratch);
    if (rc) return rc;
    QsArgs A;
    A.ngroup = ngroup;
    // as many source chunks as the slots allow, each of at least QS_CHUNK_MIN groups
    int nchunk = (ngroup + QS_CHUNK_MIN - 1) / QS_CHUNK_MIN;
    nchunk = nchunk < QS_SLOTS / ngroup ? nchunk : QS_SLOTS / ngroup;
    if (nchunk < 1) nchunk = 1;
    A.chunk_groups = (ngroup + nchunk - 1) / nchunk;
    A.nchunk = (ngroup + A.chunk_groups - 1) / A.chunk_groups;
    A.x = x; A.crg = crg; A.g_start = g_start; A.g_atoms = g_atoms; A.g_switch = g_switch; A.g_flags = g_flags;
    for (int k = 0; k < 3; ++k) A.origin[k] = origin[k];
    A.drc2_pp = rc_pp * rc_pp; A.drc2_pw = rc_pw * rc_pw; A.drc2_ww = rc_ww * rc_ww; A.drc2_lrf = rc_lrf * rc_lrf;
    A.rc2_pp = (float)A.drc2_pp; A.rc2_pw = (float)A.drc2_pw; A.rc2_ww = (float)A.drc2_ww; A.rc2_lrf = (float)A.drc2_lrf;
    A.lrf43 = lrf43; A.near_count = near_count;
    cudaStream_t st = (cudaStream_t)stream;
    dim3 grid((ngroup + QG_BLOCK - 1) / QG_BLOCK, A.nchunk);
    k_scan_static<<<grid, QG_BLOCK, 0, st>>>(A, scratch);
    k_scan_static_reduce<<<(ngroup * 32 + 127) / 128, 128, 0, st>>>(A, scratch);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return qgpu_fail(QGPU_E_CUDA, "qgpu_lrf_scan_static launch: %s", cudaGetErrorString(e));
    return 0;
}
