// qgpu_calc.cu -- qcalc-style trajectory analysis on the device.
//
// The reference's qcalc (src/qcalc.f90) reads the frames qdyn wrote to a DCD
// trajectory (src/trj.f90) and evaluates, frame by frame, the calculations of
// its calc_* modules.  Here all frames of a call are uploaded at once and each
// calculation runs over every frame in one launch:
//   * RMS deviation from the topology coordinates (calc_rms.f90 rms_calc:
//     sqrt(sum over the masked atoms of |x - x0|^2 / n), no fitting);
//   * distances, angles and torsions (calc_geom.f90 dist_calc / angle_calc /
//     torsion_calc, FP64, angles in degrees);
//   * radial distribution counts between two atom masks (calc_rdf.f90
//     RDF_calc: every pair of a mask-1 atom and a different mask-2 atom; the
//     distance in single precision and the bin index dist/radius*Nbins + 1 in
//     double, as the reference's real/real(8) mix; minimum image in a box);
//   * centre of mass of a mask (calc_com.f90 COM_calc);
//   * RMS fluctuation of a mask (calc_rmsf.f90 RMSF_calc): per atom the
//     running mean and mean square over the frames so far, the frame's value
//     the mean over the mask;
//   * least-squares fit of the solute onto the topology coordinates
//     (calc_fit.f90 fit_calc / LSQSTR): mass-weighted superposition of a mask;
//     the centres and correlation matrices of all frames on the device, the
//     rotation from each frame's six-dimensional eigenproblem on the host, and
//     the rotation of every solute atom of every frame on the device.
// Sums run in FP64 with a fixed reduction order (deterministic); RDF bins are
// integer counts.
#include <math.h>

#include <algorithm>
#include <vector>

#include "qgpu_internal.cuh"

namespace {

#define QC_T 256

struct DevBuf {
    std::vector<void *> p;
    ~DevBuf() { for (void *q : p) cudaFree(q); }
    template <class T>
    cudaError_t up(const T *h, size_t n, T **d) {
        cudaError_t e = cudaMalloc((void **)d, (n ? n : 1) * sizeof(T));
        if (e != cudaSuccess) return e;
        p.push_back(*d);
        return n ? cudaMemcpy(*d, h, n * sizeof(T), cudaMemcpyHostToDevice) : cudaSuccess;
    }
    template <class T>
    cudaError_t zero(size_t n, T **d) {
        cudaError_t e = cudaMalloc((void **)d, (n ? n : 1) * sizeof(T));
        if (e != cudaSuccess) return e;
        p.push_back(*d);
        return cudaMemset(*d, 0, (n ? n : 1) * sizeof(T));
    }
};

// block sum of one double per thread in a fixed tree order
__device__ double block_sum(double v, double *sh) {
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    const double r = sh[0];
    __syncthreads();
    return r;
}

// RMSF_calc (calc_rmsf.f90:56-80): one thread per masked atom, frames in
// order.  The running mean takes the reference's update x0 <- x0 (1 - 1/n) +
// x/n, the squares a running sum; after frame n the atom's fluctuation is
// sqrt(1/n sum_k x2_k - sum_k x0_k^2), stored as scr[f * nmask + k].  Each
// operation is rounded on its own, in the reference's order (no fused
// multiply-add): the difference of the two sums is exactly zero at the first
// frame, as in the reference, instead of a rounding residue of either sign.
__global__ void k_calc_rmsf_atoms(const double *fr, int natom, int nframes, const int *mask, int nmask, double *scr) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nmask) return;
    const int a = mask[k];
    double x0[3] = {0.0, 0.0, 0.0}, x2[3] = {0.0, 0.0, 0.0};
    for (int f = 0; f < nframes; ++f) {
        const double n = (double)(f + 1), rn = __ddiv_rn(1.0, n);
        const double *x = fr + ((size_t)f * natom + a) * 3;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            x2[c] = __dadd_rn(x2[c], __dmul_rn(x[c], x[c]));
            x0[c] = __dadd_rn(__dmul_rn(x0[c], __dsub_rn(1.0, rn)), __ddiv_rn(x[c], n));
        }
        const double s2 = __dadd_rn(__dadd_rn(x2[0], x2[1]), x2[2]);
        const double s0 = __dadd_rn(__dadd_rn(__dmul_rn(x0[0], x0[0]), __dmul_rn(x0[1], x0[1])), __dmul_rn(x0[2], x0[2]));
        scr[(size_t)f * nmask + k] = sqrt(__dsub_rn(__dmul_rn(rn, s2), s0));
    }
}
// the frame's value: (1/nmask) * the sum over the mask, one block per frame
__global__ void k_calc_rmsf_frames(const double *scr, int nmask, double *out) {
    __shared__ double sh[QC_T];
    double v = 0.0;
    for (int k = threadIdx.x; k < nmask; k += blockDim.x) v += scr[(size_t)blockIdx.x * nmask + k];
    const double sum = block_sum(v, sh);
    if (threadIdx.x == 0) out[blockIdx.x] = 1.0 / nmask * sum;
}

// Eigenvalues (descending) and eigenvectors (columns of V) of the symmetric
// N x N matrix A by cyclic Jacobi rotations (at most 60 sweeps, stopping when
// the off-diagonal sum of squares falls below 1e-30 of the total); A is
// overwritten.  Host code: the fit's six-dimensional and the kinetic
// energy's three-dimensional eigenproblems are solved per frame on the host,
// between two device passes.
template <int N>
static void jacobi(double (&A)[N][N], double (&V)[N][N], double (&ev)[N]) {
    for (int i = 0; i < N; ++i)
        for (int j = 0; j < N; ++j) V[i][j] = i == j ? 1.0 : 0.0;
    for (int sweep = 0; sweep < 60; ++sweep) {
        double off = 0.0, tot = 0.0;
        for (int i = 0; i < N; ++i)
            for (int j = 0; j < N; ++j) {
                tot += A[i][j] * A[i][j];
                if (i != j) off += A[i][j] * A[i][j];
            }
        if (!(off > 1e-30 * tot)) break;
        for (int p = 0; p < N - 1; ++p)
            for (int q = p + 1; q < N; ++q) {
                const double apq = A[p][q];
                if (apq == 0.0) continue;
                const double app = A[p][p], aqq = A[q][q];
                const double th = (aqq - app) / (2.0 * apq);
                const double t = (th >= 0.0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
                const double c = 1.0 / sqrt(t * t + 1.0), sn = t * c;
                for (int k = 0; k < N; ++k) {
                    if (k == p || k == q) continue;
                    const double akp = A[k][p], akq = A[k][q];
                    const double np = c * akp - sn * akq, nq = sn * akp + c * akq;
                    A[k][p] = np; A[p][k] = np;
                    A[k][q] = nq; A[q][k] = nq;
                }
                A[p][p] = app - t * apq;
                A[q][q] = aqq + t * apq;
                A[p][q] = 0.0; A[q][p] = 0.0;
                for (int k = 0; k < N; ++k) {
                    const double vkp = V[k][p], vkq = V[k][q];
                    V[k][p] = c * vkp - sn * vkq;
                    V[k][q] = sn * vkp + c * vkq;
                }
            }
    }
    for (int i = 0; i < N; ++i) ev[i] = A[i][i];
    for (int i = 0; i < N - 1; ++i) {   // descending (selection sort of the pairs)
        int m = i;
        for (int j = i + 1; j < N; ++j)
            if (ev[j] > ev[m]) m = j;
        if (m != i) {
            const double e = ev[i]; ev[i] = ev[m]; ev[m] = e;
            for (int k = 0; k < N; ++k) { const double v = V[k][i]; V[k][i] = V[k][m]; V[k][m] = v; }
        }
    }
}

// LSQSTR (calc_fit.f90:188-283) from the correlation matrix U: status 0 and
// the rotation R = sum_k b_k a_k^T over the three largest eigenpairs (a; b)
// of [[0, U], [U^T, 0]] (each half scaled by sqrt 2; the third with the sign
// of det U); 1 when |det U| < 1e-9; 2 when det U < 0 and the second and third
// eigenvalues are within 1e-5.  R is the identity unless the status is 0.
static int lsq_rotation(const double (&U)[3][3], double (&R)[3][3]) {
    const double du = U[0][0] * U[1][1] * U[2][2] + U[0][2] * U[1][0] * U[2][1] + U[0][1] * U[1][2] * U[2][0] -
                      U[2][0] * U[1][1] * U[0][2] - U[2][2] * U[1][0] * U[0][1] - U[2][1] * U[1][2] * U[0][0];
    for (int r = 0; r < 3; ++r)
        for (int q = 0; q < 3; ++q) R[r][q] = r == q ? 1.0 : 0.0;
    if (fabs(du) < 1e-9) return 1;
    double A[6][6] = {}, V[6][6], ev[6];
    for (int r = 0; r < 3; ++r)
        for (int q = 0; q < 3; ++q) { A[r][3 + q] = U[r][q]; A[3 + q][r] = U[r][q]; }
    jacobi<6>(A, V, ev);
    if (du < 0.0 && fabs(ev[1] - ev[2]) < 1e-5) return 2;
    for (int r = 0; r < 3; ++r)
        for (int q = 0; q < 3; ++q) {
            double v = 0.0;
            for (int k = 0; k < 3; ++k) v += (k == 2 && du < 0.0 ? -2.0 : 2.0) * V[3 + r][k] * V[q][k];
            R[r][q] = v;
        }
    return 0;
}

// fit_calc (calc_fit.f90:86-130), first device pass, one block per frame: the
// mass-weighted centre xcm of the mask and the correlation matrix U(r, s) =
// sum over the mask of X_r XP_s, X = (x - xcm) sqrt(m), XP the topology
// coordinates treated the same way about their own centre.  cu[12 f ..]:
// xcm, then U row by row.
__global__ void k_calc_fit_corr(const double *fr, int natom, const int *mask, int nmask, const double *mass,
                                const double *xp, double *cu) {
    __shared__ double sh[QC_T];
    __shared__ double s_cm[3];
    const double *x = fr + (size_t)blockIdx.x * 3 * natom;
    double c[4] = {0.0, 0.0, 0.0, 0.0};
    for (int k = threadIdx.x; k < nmask; k += blockDim.x) {
        const int a = mask[k];
        const double m = mass[a];
        c[0] += x[3 * a] * m; c[1] += x[3 * a + 1] * m; c[2] += x[3 * a + 2] * m; c[3] += m;
    }
    double cm[4];
    for (int q = 0; q < 4; ++q) cm[q] = block_sum(c[q], sh);
    if (threadIdx.x == 0)
        for (int r = 0; r < 3; ++r) { s_cm[r] = cm[r] / cm[3]; cu[12 * (size_t)blockIdx.x + r] = s_cm[r]; }
    __syncthreads();
    double u[9];
    for (int q = 0; q < 9; ++q) u[q] = 0.0;
    for (int k = threadIdx.x; k < nmask; k += blockDim.x) {
        const int a = mask[k];
        const double sm = sqrt(mass[a]);
        double X[3];
        for (int r = 0; r < 3; ++r) X[r] = (x[3 * a + r] - s_cm[r]) * sm;
        for (int r = 0; r < 3; ++r)
            for (int q = 0; q < 3; ++q) u[3 * r + q] += X[r] * xp[3 * a + q];
    }
    for (int q = 0; q < 9; ++q) {
        const double v = block_sum(u[q], sh);
        if (threadIdx.x == 0) cu[12 * (size_t)blockIdx.x + 3 + q] = v;
    }
}
// second device pass: every solute atom X = (x - xcm) sqrt(m) becomes
// R X / sqrt(m) + xrcm (rot[12 f ..]: xcm, then R row by row); solvent
// atoms are copied
__global__ void k_calc_fit_apply(const double *fr, int natom, int nsol, const double *mass, const double *rot,
                                 const double *xrcm, double *out) {
    const double *x = fr + (size_t)blockIdx.x * 3 * natom;
    double *y = out + (size_t)blockIdx.x * 3 * natom;
    const double *f = rot + 12 * (size_t)blockIdx.x;
    for (int a = threadIdx.x; a < natom; a += blockDim.x) {
        if (a >= nsol) {
            for (int r = 0; r < 3; ++r) y[3 * a + r] = x[3 * a + r];
            continue;
        }
        const double sm = sqrt(mass[a]);
        double X[3];
        for (int r = 0; r < 3; ++r) X[r] = (x[3 * a + r] - f[r]) * sm;
        for (int r = 0; r < 3; ++r)
            y[3 * a + r] = (f[3 + 3 * r] * X[0] + f[4 + 3 * r] * X[1] + f[5 + 3 * r] * X[2]) / sm + xrcm[r];
    }
}

// COM_KE_calc (calc_com_ke.f90:156-298), first device pass, one block per
// frame f: with the masses m of the mask and M their sum, the centre c of
// frame f, the centre p of the frame before (of frame f itself at f = 0,
// where the reference's previous coordinates are the current ones), and the
// inertia sums of rel = x - c: Ixx = sum m (y^2 + z^2), Iyy = sum m (x^2 +
// z^2), Izz = sum m (y^2 + x^2), Ixy = -sum y x m, Ixz = -sum x z m, Iyz =
// -sum y z m.  ci[13 f ..]: c, p, Ixx, Ixy, Iyy, Ixz, Iyz, Izz, M.
__global__ void k_calc_comke_inertia(const double *fr, int natom, const int *mask, int nmask, const double *mass,
                                     double *ci) {
    __shared__ double sh[QC_T];
    __shared__ double s_c[3];
    const int f = blockIdx.x;
    const double *x = fr + (size_t)f * 3 * natom;
    const double *xp = fr + (size_t)(f > 0 ? f - 1 : 0) * 3 * natom;
    double c[7] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int k = threadIdx.x; k < nmask; k += blockDim.x) {
        const int a = mask[k];
        const double m = mass[a];
        for (int r = 0; r < 3; ++r) { c[r] += x[3 * a + r] * m; c[3 + r] += xp[3 * a + r] * m; }
        c[6] += m;
    }
    double t[7];
    for (int q = 0; q < 7; ++q) t[q] = block_sum(c[q], sh);
    double *o = ci + 13 * (size_t)f;
    if (threadIdx.x == 0) {
        for (int r = 0; r < 3; ++r) { s_c[r] = t[r] / t[6]; o[r] = s_c[r]; o[3 + r] = t[3 + r] / t[6]; }
        o[12] = t[6];
    }
    __syncthreads();
    double I[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int k = threadIdx.x; k < nmask; k += blockDim.x) {
        const int a = mask[k];
        const double m = mass[a];
        const double rx = x[3 * a] - s_c[0], ry = x[3 * a + 1] - s_c[1], rz = x[3 * a + 2] - s_c[2];
        I[0] += (ry * ry + rz * rz) * m;
        I[1] += ry * rx * m;
        I[2] += (rx * rx + rz * rz) * m;
        I[3] += rx * rz * m;
        I[4] += ry * rz * m;
        I[5] += (ry * ry + rx * rx) * m;
    }
    for (int q = 0; q < 6; ++q) {
        const double v = block_sum(I[q], sh);
        if (threadIdx.x == 0) o[6 + q] = (q == 1 || q == 3 || q == 4) ? -v : v;
    }
}

// COM_KE_calc second pass, one block per frame: the velocity v = (rel -
// rel')/dt of every mask atom relative to its frame's centre (rel' about
// the previous frame's centre), and for each principal axis e_j of the
// inertia tensor (ax[12 f + 3 j ..], from the host) the angular momentum
// L_j = sum m (rad_j x v), rad_j = rel - (e_j . rel) e_j.  lm[9 f + 3 j ..].
__global__ void k_calc_comke_angmom(const double *fr, int natom, const int *mask, int nmask, const double *mass,
                                    const double *ci, const double *ax, double dt, double *lm) {
    __shared__ double sh[QC_T];
    const int f = blockIdx.x;
    const double *x = fr + (size_t)f * 3 * natom;
    const double *xp = fr + (size_t)(f > 0 ? f - 1 : 0) * 3 * natom;
    const double *c = ci + 13 * (size_t)f;
    const double *e = ax + 12 * (size_t)f;
    double L[9];
    for (int q = 0; q < 9; ++q) L[q] = 0.0;
    for (int k = threadIdx.x; k < nmask; k += blockDim.x) {
        const int a = mask[k];
        const double m = mass[a];
        double rel[3], v[3];
        for (int r = 0; r < 3; ++r) {
            rel[r] = x[3 * a + r] - c[r];
            v[r] = (rel[r] - (xp[3 * a + r] - c[3 + r])) / dt;
        }
        for (int j = 0; j < 3; ++j) {
            const double dp = e[3 * j] * rel[0] + e[3 * j + 1] * rel[1] + e[3 * j + 2] * rel[2];
            const double rx = rel[0] - dp * e[3 * j], ry = rel[1] - dp * e[3 * j + 1], rz = rel[2] - dp * e[3 * j + 2];
            L[3 * j] += ry * v[2] * m - rz * v[1] * m;
            L[3 * j + 1] += rz * v[0] * m - rx * v[2] * m;
            L[3 * j + 2] += rx * v[1] * m - ry * v[0] * m;
        }
    }
    for (int q = 0; q < 9; ++q) {
        const double s = block_sum(L[q], sh);
        if (threadIdx.x == 0) lm[9 * (size_t)f + q] = s;
    }
}

// rms_calc (calc_rms.f90): one block per frame
__global__ void k_calc_rms(const double *fr, int natom, const int *mask, int n, const double *x0, double *out) {
    __shared__ double sh[QC_T];
    const double *x = fr + (size_t)blockIdx.x * 3 * natom;
    double s = 0.0;
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const int a = mask[k];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const double d = x[3 * a + c] - x0[3 * a + c];
            s += d * d;
        }
    }
    s = block_sum(s, sh);
    if (threadIdx.x == 0) out[blockIdx.x] = sqrt(s / n);
}

// COM_calc (calc_com.f90): one block per frame, the mass-weighted mean
__global__ void k_calc_com(const double *fr, int natom, const int *mask, int n, const double *mass, double *out) {
    __shared__ double sh[QC_T];
    const double *x = fr + (size_t)blockIdx.x * 3 * natom;
    double c[3] = {0.0, 0.0, 0.0}, m = 0.0;
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const int a = mask[k];
        m += mass[a];
#pragma unroll
        for (int d = 0; d < 3; ++d) c[d] += x[3 * a + d] * mass[a];
    }
    const double mt = block_sum(m, sh);
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const double s = block_sum(c[d], sh);
        if (threadIdx.x == 0) out[3 * blockIdx.x + d] = s / mt;
    }
}

// dist_calc / angle_calc / torsion_calc (calc_geom.f90): one thread per
// (frame, measurement); kind 2 distance (A), 3 angle, 4 torsion (degrees)
__global__ void k_calc_geom(const double *fr, int natom, int nframes, int nmeas, const int *atoms, const int *kind,
                            double *out) {
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= nframes * nmeas) return;
    const int f = id / nmeas, m = id % nmeas;
    const double *x = fr + (size_t)f * 3 * natom;
    const int *at = atoms + 4 * m;
    const double pi = 4.0 * atan(1.0);
    auto diff = [&](int a, int b, double (&r)[3]) {
#pragma unroll
        for (int c = 0; c < 3; ++c) r[c] = x[3 * a + c] - x[3 * b + c];
    };
    auto dot = [](const double (&a)[3], const double (&b)[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; };
    double v = 0.0;
    if (kind[m] == 2) {
        double rji[3];
        diff(at[0], at[1], rji);
        v = sqrt(dot(rji, rji));
    } else if (kind[m] == 3) {
        double rji[3], rjk[3];
        diff(at[0], at[1], rji);
        diff(at[2], at[1], rjk);
        double scp = dot(rji, rjk) / sqrt(dot(rji, rji) * dot(rjk, rjk));
        scp = fmin(fmax(scp, -1.0), 1.0);
        v = acos(scp) * 180.0 / pi;
    } else {
        double rji[3], rjk[3], rkl[3], rnj[3], rnk[3];
        diff(at[0], at[1], rji);
        diff(at[2], at[1], rjk);
        diff(at[3], at[2], rkl);
        rnj[0] = rji[1] * rjk[2] - rji[2] * rjk[1];
        rnj[1] = rji[2] * rjk[0] - rji[0] * rjk[2];
        rnj[2] = rji[0] * rjk[1] - rji[1] * rjk[0];
        rnk[0] = -rjk[1] * rkl[2] + rjk[2] * rkl[1];
        rnk[1] = -rjk[2] * rkl[0] + rjk[0] * rkl[2];
        rnk[2] = -rjk[0] * rkl[1] + rjk[1] * rkl[0];
        double scp = dot(rnj, rnk) / sqrt(dot(rnj, rnj) * dot(rnk, rnk));
        scp = fmin(fmax(scp, -1.0), 1.0);
        double phi = acos(scp);
        const double sgn = rjk[0] * (rnj[1] * rnk[2] - rnj[2] * rnk[1]) + rjk[1] * (rnj[2] * rnk[0] - rnj[0] * rnk[2]) +
                           rjk[2] * (rnj[0] * rnk[1] - rnj[1] * rnk[0]);
        if (sgn < 0) phi = -phi;
        v = phi * 180.0 / pi;
    }
    out[(size_t)f * nmeas + m] = v;
}

// RDF_calc (calc_rdf.f90): the single-precision pair distance of the
// reference (function r, FP64 difference rounded to real(4), minimum image
// in double and rounded again, dot product and sqrt in real(4) without
// contraction) and its bin dist/radius*Nbins + 1 in double.
__device__ __forceinline__ float rdf_comp(double xa, double xb, double box) {
    float d = (float)(xa - xb);
    if (box > 0.0) d = (float)((double)d - box * round((double)d / box));
    return d;
}
// one thread per (frame, mask-1 atom), mask 2 staged through shared memory;
// counts gathered in shared bins, then added to the global bins (integers)
__global__ void k_calc_rdf(const double *fr, int natom, const int *m1, int n1, const int *m2, int n2, double radius,
                           int nbins, double bx, double by, double bz, int use_box, unsigned long long *bins) {
    extern __shared__ unsigned int sb[];   // nbins counters
    __shared__ double s2[QC_T][3];
    __shared__ int si[QC_T];
    const int f = blockIdx.y;
    const double *x = fr + (size_t)f * 3 * natom;
    for (int k = threadIdx.x; k < nbins; k += blockDim.x) sb[k] = 0u;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool on = i < n1;
    const int a = on ? m1[i] : 0;
    const double xa = on ? x[3 * a] : 0.0, ya = on ? x[3 * a + 1] : 0.0, za = on ? x[3 * a + 2] : 0.0;
    for (int j0 = 0; j0 < n2; j0 += blockDim.x) {
        __syncthreads();
        const int jj = j0 + threadIdx.x;
        if (jj < n2) {
            const int b = m2[jj];
            si[threadIdx.x] = b;
            s2[threadIdx.x][0] = x[3 * b]; s2[threadIdx.x][1] = x[3 * b + 1]; s2[threadIdx.x][2] = x[3 * b + 2];
        }
        __syncthreads();
        const int nj = min((int)blockDim.x, n2 - j0);
        if (!on) continue;
        for (int j = 0; j < nj; ++j) {
            if (si[j] == a) continue;
            const float d1 = rdf_comp(xa, s2[j][0], use_box ? bx : 0.0);
            const float d2 = rdf_comp(ya, s2[j][1], use_box ? by : 0.0);
            const float d3 = rdf_comp(za, s2[j][2], use_box ? bz : 0.0);
            const float r2 = __fadd_rn(__fadd_rn(__fmul_rn(d1, d1), __fmul_rn(d2, d2)), __fmul_rn(d3, d3));
            const float dist = __fsqrt_rn(r2);
            if ((double)dist < radius) {
                const int bin = (int)((double)dist / radius * (double)nbins + 1.0) - 1;
                if (bin >= 0 && bin < nbins) atomicAdd(&sb[bin], 1u);
            }
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < nbins; k += blockDim.x)
        if (sb[k]) atomicAdd(&bins[k], (unsigned long long)sb[k]);
}

// nb_calc_lists (calc_nb.f90:257-328): block (c, f) sums the pairs of chunk
// c at frame f, pairs [ch[c].x, ch[c].y) of one list (a chunk never spans
// two lists), the per-state products stored pair-major (AA[p*S + s]).  A
// pair at r = 0 adds nothing.
#define QC_NBCH 2048
__global__ void k_calc_nb(const double *fr, int natom, const int2 *pairs, const longlong2 *ch, int S, const double *lam,
                          const double *AA, const double *BB, const double *qq, int arith, double *part) {
    __shared__ double sh[QC_T];
    const int f = blockIdx.y;
    const double *x = fr + (size_t)f * 3 * natom;
    const long long p0 = ch[blockIdx.x].x, p1 = ch[blockIdx.x].y;
    double lj = 0.0, el = 0.0;
    for (long long p = p0 + threadIdx.x; p < p1; p += blockDim.x) {
        const int2 a = pairs[p];
        const double dx = x[3 * a.x] - x[3 * a.y], dy = x[3 * a.x + 1] - x[3 * a.y + 1];
        const double dz = x[3 * a.x + 2] - x[3 * a.y + 2];
        const double r = sqrt(dx * dx + dy * dy + dz * dz);
        if (r == 0.0) continue;
        const double invr = 1.0 / r;
        const double invr2 = invr * invr;
        const double invr6 = invr2 * invr2 * invr2;
        const double invr12 = invr6 * invr6;
        for (int s = 0; s < S; ++s) {
            const double A = AA[p * S + s], B = BB[p * S + s];
            double v;
            if (arith) {
                const double A2 = A * A, A6 = A2 * A2 * A2;
                v = sqrt(B) * A6 * invr6 * (A6 * invr6 - 2.0);
            } else {
                v = A * invr12 - B * invr6;
            }
            lj += lam[s] * v;
            el += lam[s] * (qq[p * S + s] * invr);
        }
    }
    lj = block_sum(lj, sh);
    el = block_sum(el, sh);
    if (threadIdx.x == 0) {
        part[2 * ((size_t)f * gridDim.x + blockIdx.x)] = lj;
        part[2 * ((size_t)f * gridDim.x + blockIdx.x) + 1] = el;
    }
}

// one thread per (frame, list, term): the list's chunk sums in chunk order
// (chunks c0[l] .. c0[l+1]-1)
__global__ void k_calc_nb_lists(const double *part, const int *c0, int nch, int nlist, int nframes, double *out) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 2LL * nlist * nframes) return;
    const int e = (int)(t & 1);
    const long long fl = t >> 1;
    const int f = (int)(fl / nlist), l = (int)(fl % nlist);
    double v = 0.0;
    for (int c = c0[l]; c < c0[l + 1]; ++c) v += part[2 * ((size_t)f * nch + c) + e];
    out[t] = v;
}

int check_atoms(const int32_t *a, int n, int natom) {
    for (int k = 0; k < n; ++k)
        if (a[k] < 0 || a[k] >= natom) return 1;
    return 0;
}

#define CKC(call)                                                                                     \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess) return qgpu_fail(QGPU_E_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

}  // namespace

extern "C" {

int qgpu_calc_rms(const double *frames, int32_t nframes, int32_t natom, const int32_t *mask, int32_t nmask,
                  const double *xref, double *out) {
    if (!frames || nframes < 1 || natom < 1 || !mask || nmask < 1 || !xref || !out || check_atoms(mask, nmask, natom))
        return qgpu_fail(QGPU_E_INVALID, "qgpu_calc_rms: bad arguments");
    DevBuf B;
    double *fr, *x0, *o;
    int *m;
    CKC(B.up(frames, (size_t)nframes * 3 * natom, &fr));
    CKC(B.up(xref, (size_t)3 * natom, &x0));
    CKC(B.up(mask, (size_t)nmask, &m));
    CKC(B.zero((size_t)nframes, &o));
    k_calc_rms<<<nframes, QC_T>>>(fr, natom, m, nmask, x0, o);
    CKC(cudaGetLastError());
    CKC(cudaMemcpy(out, o, (size_t)nframes * sizeof(double), cudaMemcpyDeviceToHost));
    return 0;
}

int qgpu_calc_rmsf(const double *frames, int32_t nframes, int32_t natom, const int32_t *mask, int32_t nmask,
                   double *out) {
    if (!frames || nframes < 1 || natom < 1 || !mask || nmask < 1 || !out || check_atoms(mask, nmask, natom))
        return qgpu_fail(QGPU_E_INVALID, "qgpu_calc_rmsf: bad arguments");
    DevBuf B;
    double *fr, *scr, *o;
    int *m;
    CKC(B.up(frames, (size_t)nframes * 3 * natom, &fr));
    CKC(B.up(mask, (size_t)nmask, &m));
    CKC(B.zero((size_t)nframes * nmask, &scr));
    CKC(B.zero((size_t)nframes, &o));
    k_calc_rmsf_atoms<<<(nmask + QC_T - 1) / QC_T, QC_T>>>(fr, natom, nframes, m, nmask, scr);
    CKC(cudaGetLastError());
    k_calc_rmsf_frames<<<nframes, QC_T>>>(scr, nmask, o);
    CKC(cudaGetLastError());
    CKC(cudaMemcpy(out, o, (size_t)nframes * sizeof(double), cudaMemcpyDeviceToHost));
    return 0;
}

int qgpu_calc_fit(const double *frames, int32_t nframes, int32_t natom, int32_t nsol, const int32_t *mask,
                  int32_t nmask, const double *mass, const double *xref, double *out, int32_t *status) {
    if (!frames || nframes < 1 || natom < 1 || nsol < 1 || nsol > natom || !mask || nmask < 1 || !mass || !xref ||
        !out || !status || check_atoms(mask, nmask, nsol))
        return qgpu_fail(QGPU_E_INVALID, "qgpu_calc_fit: bad arguments");
    // the reference frame (fit_make_ref, calc_fit.f90:133-155): its centre of
    // mass over the mask and every solute atom's (xtop - xrcm) sqrt(m)
    double xrcm[3] = {0.0, 0.0, 0.0}, tm = 0.0;
    for (int k = 0; k < nmask; ++k) {
        const int a = mask[k];
        for (int r = 0; r < 3; ++r) xrcm[r] += xref[3 * a + r] * mass[a];
        tm += mass[a];
    }
    if (!(tm > 0.0)) return qgpu_fail(QGPU_E_INVALID, "qgpu_calc_fit: zero mass");
    for (int r = 0; r < 3; ++r) xrcm[r] = xrcm[r] / tm;
    std::vector<double> xp(3 * (size_t)natom, 0.0);
    for (int a = 0; a < nsol; ++a)
        for (int r = 0; r < 3; ++r) xp[3 * a + r] = (xref[3 * a + r] - xrcm[r]) * sqrt(mass[a]);
    DevBuf B;
    double *fr, *ms, *xpd, *rc, *o, *cu, *rot;
    int *m;
    CKC(B.up(frames, (size_t)nframes * 3 * natom, &fr));
    CKC(B.up(mass, (size_t)natom, &ms));
    CKC(B.up(xp.data(), xp.size(), &xpd));
    CKC(B.up(xrcm, (size_t)3, &rc));
    CKC(B.up(mask, (size_t)nmask, &m));
    CKC(B.zero((size_t)nframes * 3 * natom, &o));
    CKC(B.zero((size_t)nframes * 12, &cu));
    k_calc_fit_corr<<<nframes, QC_T>>>(fr, natom, m, nmask, ms, xpd, cu);
    CKC(cudaGetLastError());
    // the per-frame 6x6 eigenproblems on the host
    std::vector<double> h((size_t)nframes * 12);
    CKC(cudaMemcpy(h.data(), cu, h.size() * sizeof(double), cudaMemcpyDeviceToHost));
    for (int f = 0; f < nframes; ++f) {
        double U[3][3], R[3][3];
        for (int r = 0; r < 3; ++r)
            for (int q = 0; q < 3; ++q) U[r][q] = h[12 * (size_t)f + 3 + 3 * r + q];
        status[f] = lsq_rotation(U, R);
        for (int r = 0; r < 3; ++r)
            for (int q = 0; q < 3; ++q) h[12 * (size_t)f + 3 + 3 * r + q] = R[r][q];
    }
    CKC(B.up(h.data(), h.size(), &rot));
    k_calc_fit_apply<<<nframes, QC_T>>>(fr, natom, nsol, ms, rot, rc, o);
    CKC(cudaGetLastError());
    CKC(cudaMemcpy(out, o, (size_t)nframes * 3 * natom * sizeof(double), cudaMemcpyDeviceToHost));
    return 0;
}

int qgpu_calc_com_ke(const double *frames, int32_t nframes, int32_t natom, const int32_t *mask, int32_t nmask,
                     const double *mass, double frame_length, double *out) {
    if (!frames || nframes < 1 || natom < 1 || !mask || nmask < 1 || !mass || !(frame_length > 0) || !out ||
        check_atoms(mask, nmask, natom))
        return qgpu_fail(QGPU_E_INVALID, "qgpu_calc_com_ke: bad arguments");
    // g/mol A^2/fs^2 to kcal/mol: the reference declares the factor 2390.0574
    // as an integer parameter (calc_com_ke.f90:33), so it is 2390
    const double conv = 2390.0;
    DevBuf B;
    double *fr, *ms, *ci, *ax, *lm;
    int *m;
    CKC(B.up(frames, (size_t)nframes * 3 * natom, &fr));
    CKC(B.up(mass, (size_t)natom, &ms));
    CKC(B.up(mask, (size_t)nmask, &m));
    CKC(B.zero((size_t)nframes * 13, &ci));
    CKC(B.zero((size_t)nframes * 9, &lm));
    k_calc_comke_inertia<<<nframes, QC_T>>>(fr, natom, m, nmask, ms, ci);
    CKC(cudaGetLastError());
    std::vector<double> h((size_t)nframes * 13), e((size_t)nframes * 12), iv((size_t)nframes * 3);
    CKC(cudaMemcpy(h.data(), ci, h.size() * sizeof(double), cudaMemcpyDeviceToHost));
    for (int f = 0; f < nframes; ++f) {
        // EIGEN of the packed (Ixx, Ixy, Iyy, Ixz, Iyz, Izz): principal moments
        // and axes (calc_com_ke.f90:226-232)
        const double *I = &h[13 * (size_t)f + 6];
        double A[3][3] = {{I[0], I[1], I[3]}, {I[1], I[2], I[4]}, {I[3], I[4], I[5]}}, V[3][3], ev[3];
        jacobi<3>(A, V, ev);
        for (int j = 0; j < 3; ++j) {
            iv[3 * (size_t)f + j] = ev[j];
            for (int r = 0; r < 3; ++r) e[12 * (size_t)f + 3 * j + r] = V[r][j];
        }
    }
    CKC(B.up(e.data(), e.size(), &ax));
    k_calc_comke_angmom<<<nframes, QC_T>>>(fr, natom, m, nmask, ms, ci, ax, frame_length, lm);
    CKC(cudaGetLastError());
    std::vector<double> L((size_t)nframes * 9);
    CKC(cudaMemcpy(L.data(), lm, L.size() * sizeof(double), cudaMemcpyDeviceToHost));
    for (int f = 0; f < nframes; ++f) {
        const double *c = &h[13 * (size_t)f];
        double rot = 0.0;
        for (int j = 0; j < 3; ++j) {
            const double *l = &L[9 * (size_t)f + 3 * j];
            rot += (l[0] * l[0] + l[1] * l[1] + l[2] * l[2]) / (2.0 * iv[3 * (size_t)f + j]) * conv;
        }
        const double d0 = c[3] - c[0], d1 = c[4] - c[1], d2 = c[5] - c[2];
        out[2 * f] = 0.5 * c[12] * (d0 * d0 + d1 * d1 + d2 * d2) / (frame_length * frame_length) * conv;
        out[2 * f + 1] = rot;
    }
    return 0;
}

int qgpu_calc_com(const double *frames, int32_t nframes, int32_t natom, const int32_t *mask, int32_t nmask,
                  const double *mass, double *out) {
    if (!frames || nframes < 1 || natom < 1 || !mask || nmask < 1 || !mass || !out || check_atoms(mask, nmask, natom))
        return qgpu_fail(QGPU_E_INVALID, "qgpu_calc_com: bad arguments");
    DevBuf B;
    double *fr, *ms, *o;
    int *m;
    CKC(B.up(frames, (size_t)nframes * 3 * natom, &fr));
    CKC(B.up(mass, (size_t)natom, &ms));
    CKC(B.up(mask, (size_t)nmask, &m));
    CKC(B.zero((size_t)3 * nframes, &o));
    k_calc_com<<<nframes, QC_T>>>(fr, natom, m, nmask, ms, o);
    CKC(cudaGetLastError());
    CKC(cudaMemcpy(out, o, (size_t)3 * nframes * sizeof(double), cudaMemcpyDeviceToHost));
    return 0;
}

int qgpu_calc_geom(const double *frames, int32_t nframes, int32_t natom, int32_t nmeas, const int32_t *atoms,
                   const int32_t *kind, double *out) {
    if (!frames || nframes < 1 || natom < 1 || nmeas < 1 || !atoms || !kind || !out)
        return qgpu_fail(QGPU_E_INVALID, "qgpu_calc_geom: bad arguments");
    for (int m = 0; m < nmeas; ++m) {
        if (kind[m] < 2 || kind[m] > 4) return qgpu_fail(QGPU_E_INVALID, "qgpu_calc_geom: kind %d", kind[m]);
        if (check_atoms(atoms + 4 * m, kind[m], natom)) return qgpu_fail(QGPU_E_INVALID, "qgpu_calc_geom: atom index");
    }
    std::vector<int32_t> at((size_t)4 * nmeas);
    for (int m = 0; m < nmeas; ++m)
        for (int k = 0; k < 4; ++k) at[4 * m + k] = k < kind[m] ? atoms[4 * m + k] : 0;
    DevBuf B;
    double *fr, *o;
    int *a, *kd;
    CKC(B.up(frames, (size_t)nframes * 3 * natom, &fr));
    CKC(B.up(at.data(), at.size(), &a));
    CKC(B.up(kind, (size_t)nmeas, &kd));
    CKC(B.zero((size_t)nframes * nmeas, &o));
    const int n = nframes * nmeas;
    k_calc_geom<<<(n + QC_T - 1) / QC_T, QC_T>>>(fr, natom, nframes, nmeas, a, kd, o);
    CKC(cudaGetLastError());
    CKC(cudaMemcpy(out, o, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost));
    return 0;
}

int qgpu_calc_rdf(const double *frames, int32_t nframes, int32_t natom, const int32_t *mask1, int32_t n1,
                  const int32_t *mask2, int32_t n2, double radius, int32_t nbins, const double *box, int64_t *counts) {
    if (!frames || nframes < 1 || natom < 1 || !mask1 || n1 < 1 || !mask2 || n2 < 1 || !(radius > 0) || nbins < 1 ||
        nbins > 8192 || !counts || check_atoms(mask1, n1, natom) || check_atoms(mask2, n2, natom) ||
        nframes > 65535)
        return qgpu_fail(QGPU_E_INVALID, "qgpu_calc_rdf: bad arguments");
    DevBuf B;
    double *fr;
    int *a, *b;
    unsigned long long *bins;
    CKC(B.up(frames, (size_t)nframes * 3 * natom, &fr));
    CKC(B.up(mask1, (size_t)n1, &a));
    CKC(B.up(mask2, (size_t)n2, &b));
    CKC(B.zero((size_t)nbins, &bins));
    dim3 grid((n1 + QC_T - 1) / QC_T, nframes);
    k_calc_rdf<<<grid, QC_T, (size_t)nbins * sizeof(unsigned int)>>>(fr, natom, a, n1, b, n2, radius, nbins,
                                                                     box ? box[0] : 0.0, box ? box[1] : 0.0,
                                                                     box ? box[2] : 0.0, box ? 1 : 0, bins);
    CKC(cudaGetLastError());
    std::vector<unsigned long long> h(nbins);
    CKC(cudaMemcpy(h.data(), bins, (size_t)nbins * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
    for (int k = 0; k < nbins; ++k) counts[k] = (int64_t)h[k];
    return 0;
}

int qgpu_calc_nb(const double *frames, int32_t nframes, int32_t natom, int32_t nlist, const int64_t *list_start,
                 const int32_t *pairs, int32_t nstates, const double *lambdas, const double *AA, const double *BB,
                 const double *qq, int32_t arith, double *out) {
    if (!frames || nframes < 1 || nframes > 65535 || natom < 1 || nlist < 1 || !list_start || nstates < 1 ||
        nstates > QGPU_MAX_STATES || !lambdas || !out || (arith != 0 && arith != 1))
        return qgpu_fail(QGPU_E_INVALID, "qgpu_calc_nb: bad arguments");
    if (list_start[0] != 0) return qgpu_fail(QGPU_E_INVALID, "qgpu_calc_nb: list_start[0] must be 0");
    for (int l = 0; l < nlist; ++l)
        if (list_start[l + 1] < list_start[l]) return qgpu_fail(QGPU_E_INVALID, "qgpu_calc_nb: list_start decreases");
    const int64_t npair = list_start[nlist];
    if (npair > ((int64_t)1 << 40) || (npair > 0 && (!pairs || !AA || !BB || !qq)))
        return qgpu_fail(QGPU_E_INVALID, "qgpu_calc_nb: bad pair arrays");
    for (int64_t k = 0; k < 2 * npair; ++k)
        if (pairs[k] < 0 || pairs[k] >= natom) return qgpu_fail(QGPU_E_INVALID, "qgpu_calc_nb: atom out of range");
    // chunks of at most QC_NBCH pairs, none spanning two lists
    std::vector<long long> chs;
    std::vector<int> c0((size_t)nlist + 1, 0);
    for (int l = 0; l < nlist; ++l) {
        c0[l] = (int)(chs.size() / 2);
        for (int64_t p = list_start[l]; p < list_start[l + 1]; p += QC_NBCH) {
            chs.push_back(p);
            chs.push_back(std::min<int64_t>(list_start[l + 1], p + QC_NBCH));
        }
        if (chs.size() / 2 > 0x7fffffffu) return qgpu_fail(QGPU_E_INVALID, "qgpu_calc_nb: lists too long");
    }
    const int nch = (int)(chs.size() / 2);
    c0[nlist] = nch;
    if (nch == 0) {
        for (long long k = 0; k < 2LL * nframes * nlist; ++k) out[k] = 0.0;
        return 0;
    }
    DevBuf B;
    double *fr, *lam, *a, *b, *q, *part, *o;
    int32_t *pr;
    long long *chd;
    int *c0d;
    const size_t ns = (size_t)npair * nstates;
    CKC(B.up(frames, (size_t)nframes * 3 * natom, &fr));
    CKC(B.up(pairs, (size_t)2 * npair, &pr));
    CKC(B.up(lambdas, (size_t)nstates, &lam));
    CKC(B.up(AA, ns, &a));
    CKC(B.up(BB, ns, &b));
    CKC(B.up(qq, ns, &q));
    CKC(B.up(chs.data(), chs.size(), &chd));
    CKC(B.up(c0.data(), c0.size(), &c0d));
    CKC(B.zero((size_t)2 * nframes * nch, &part));
    CKC(B.zero((size_t)2 * nframes * nlist, &o));
    k_calc_nb<<<dim3((unsigned)nch, nframes), QC_T>>>(fr, natom, (const int2 *)pr, (const longlong2 *)chd, nstates, lam,
                                                      a, b, q, arith, part);
    CKC(cudaGetLastError());
    const long long nt = 2LL * nframes * nlist;
    k_calc_nb_lists<<<(unsigned)((nt + QC_T - 1) / QC_T), QC_T>>>(part, c0d, nch, nlist, nframes, o);
    CKC(cudaGetLastError());
    CKC(cudaMemcpy(out, o, (size_t)nt * sizeof(double), cudaMemcpyDeviceToHost));
    return 0;
}

}  // extern "C"
