// qgpu_ene.cu -- Q energy files (.en), the binary file qfep reads.
//
// Layout (Fortran unformatted sequential records, each framed by a 4-byte
// length before and after the payload, as gfortran writes them):
//   header (prep_sim_version, src/md.f90:17011-17015), arrays = 1:
//     int32 canary (1337 = double precision), arrays (1), totresid (1),
//     types(1) (NOGC = 3, misc.f90:36), numres(1) (1), resid(1) (-1),
//     gcnum(1) (-1), char[80] version
//   per frame (put_ene, src/nrgy.f90:94-123):
//     nstates records: int32 state (1-based), f64 lambda, total, q%bond,
//       q%angle, q%torsion, q%improper, qx%el, qx%vdw, qq%el, qq%vdw, qp%el,
//       qp%vdw, qw%el, qw%vdw, restraint
//     one OFFD record: per coupling int32 i, int32 j, f64 Hij, f64 rkl (empty
//       when there are none)
// qdyn writes a frame at every nonzero multiple of iene_cycle
// (md_run, src/md.f90:6630-6633).  Host code only.
#include <stdio.h>
#include <string.h>

#include <vector>

#include "qgpu_internal.cuh"

namespace {

bool put_record(FILE *f, const void *payload, int32_t n) {
    return fwrite(&n, 4, 1, f) == 1 && (n == 0 || fwrite(payload, 1, (size_t)n, f) == (size_t)n) &&
           fwrite(&n, 4, 1, f) == 1;
}

struct Rec {
    std::vector<unsigned char> b;
    void i32(int32_t v) { const unsigned char *p = (const unsigned char *)&v; b.insert(b.end(), p, p + 4); }
    void f64(double v) { const unsigned char *p = (const unsigned char *)&v; b.insert(b.end(), p, p + 8); }
};

}  // namespace

// header record; returns 0 or QGPU_E_INVALID
int qgpu_ene_write_header(FILE *f, const char *version) {
    Rec r;
    r.i32(1337); r.i32(1); r.i32(1); r.i32(3); r.i32(1); r.i32(-1); r.i32(-1);
    char v[80];
    memset(v, ' ', sizeof v);
    const char *src = version ? version : "";
    memcpy(v, src, strnlen(src, sizeof v));
    r.b.insert(r.b.end(), v, v + 80);
    return put_record(f, r.b.data(), (int32_t)r.b.size()) ? 0 : QGPU_E_INVALID;
}

// one frame: nstates state records and the OFFD record
int qgpu_ene_write_frame(FILE *f, int32_t nstates, const qgpu_qenergy *EQ, int32_t noffd, const int32_t *offd_ij,
                         const double *offd_Hr) {
    for (int s = 0; s < nstates; ++s) {
        const qgpu_qenergy &q = EQ[s];
        Rec r;
        r.i32(s + 1);
        const double v[15] = {q.lambda, q.total, q.q_bond, q.q_angle, q.q_torsion, q.q_improper, q.qx_el, q.qx_vdw,
                              q.qq_el, q.qq_vdw, q.qp_el, q.qp_vdw, q.qw_el, q.qw_vdw, q.restraint};
        for (double x : v) r.f64(x);
        if (!put_record(f, r.b.data(), (int32_t)r.b.size())) return QGPU_E_INVALID;
    }
    Rec o;
    for (int k = 0; k < noffd; ++k) {
        o.i32(offd_ij[2 * k]); o.i32(offd_ij[2 * k + 1]);
        o.f64(offd_Hr[2 * k]); o.f64(offd_Hr[2 * k + 1]);
    }
    return put_record(f, o.b.data(), (int32_t)o.b.size()) ? 0 : QGPU_E_INVALID;
}

extern "C" int qgpu_enefile_write(const char *path, int32_t nframes, int32_t nstates, const qgpu_qenergy *frames,
                                  int32_t noffd, const int32_t *offd_ij, const double *offd_Hr) {
    if (!path || nframes < 0 || nstates < 1 || nstates > QGPU_MAX_STATES || (nframes && !frames) || noffd < 0 ||
        (noffd && (!offd_ij || !offd_Hr)))
        return qgpu_fail(QGPU_E_INVALID, "qgpu_enefile_write: bad arguments");
    FILE *f = fopen(path, "wb");
    if (!f) return qgpu_fail(QGPU_E_INVALID, "qgpu_enefile_write: cannot open %s", path);
    int rc = qgpu_ene_write_header(f, "5.06 (qsource_gb300)");
    for (int k = 0; k < nframes && !rc; ++k)
        rc = qgpu_ene_write_frame(f, nstates, frames + (size_t)k * nstates, noffd, offd_ij,
                                  offd_Hr ? offd_Hr + (size_t)k * 2 * noffd : nullptr);
    if (fclose(f) != 0 && !rc) rc = QGPU_E_INVALID;
    if (rc) return qgpu_fail(rc, "qgpu_enefile_write: write to %s failed", path);
    return 0;
}
