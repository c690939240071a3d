/*
 * qgpu_drop_in.c -- a plain C host of the engine's C-ABI (include/qgpu.h),
 * making qdyn's own call sequence for one step-0 evaluation:
 *
 *   qgpu_create          (start-up, after src/qdyn.f90:110-124)
 *   qgpu_build_lists     (make_pair_lists, src/md.f90:6505)
 *   qgpu_forces          (pot_energy_nonbonds + nonbond_qq + Q/classical
 *                         bonded terms, src/md.f90:16096-16150)
 *   qgpu_shake           (shake, src/md.f90:6596)
 *
 * The system descriptor comes from a file written by the test that runs this
 * program (tests/test_c_abi.py): the bytes of a qgpu_system_desc, a table of
 * the byte offsets of its pointer fields, and the arrays those fields point
 * to, stored as offsets into the array block ("relocations").  Everything
 * after loading is plain use of the header's types and entry points.
 *
 * Usage: qgpu_drop_in <descriptor file> <shaken x out> QEL QVdW EL VdW QBND QANG QTOR QIMP BND ANG TOR IMP
 * The 12 numbers are the reference's printed step-0 values
 * (tests/basic_tests/SPH_leap-frog_berendsen_benchmark.en row 1); the program
 * exits 0 when every column rounds to the printed value and SHAKE converged
 * and shrank the constraint violations.  The shaken coordinates go to the
 * second file (3*natom doubles) for the caller to compare with the oracle: the
 * reference's SHAKE does not revisit a constraint once it met the tolerance,
 * so coupled constraints can end somewhat outside it.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "qgpu.h"

static int fail(const char *what) {
    char msg[512];
    qgpu_last_error(msg, (int32_t)sizeof msg);
    fprintf(stderr, "%s failed: %s\n", what, msg);
    return 1;
}

int main(int argc, char **argv) {
    if (argc != 15) {
        fprintf(stderr, "usage: %s desc xout QEL QVdW EL VdW QBND QANG QTOR QIMP BND ANG TOR IMP\n", argv[0]);
        return 2;
    }
    FILE *f = fopen(argv[1], "rb");
    if (!f) { perror(argv[1]); return 2; }
    char magic[8];
    unsigned long long hdr[3];   /* struct bytes, relocations, array bytes */
    if (fread(magic, 1, 8, f) != 8 || memcmp(magic, "QGPUDESC", 8) || fread(hdr, 8, 3, f) != 3) {
        fprintf(stderr, "bad descriptor file\n");
        return 2;
    }
    if (hdr[0] != sizeof(qgpu_system_desc)) {
        fprintf(stderr, "sizeof(qgpu_system_desc) = %zu here, %llu in the file\n", sizeof(qgpu_system_desc), hdr[0]);
        return 2;
    }
    qgpu_system_desc d;
    unsigned long long *rel = malloc(8 * (hdr[1] + 1));
    unsigned char *blk = malloc(hdr[2] + 8);
    if (!rel || !blk || fread(&d, 1, sizeof d, f) != sizeof d || fread(rel, 8, hdr[1], f) != hdr[1] ||
        fread(blk, 1, hdr[2], f) != hdr[2]) {
        fprintf(stderr, "short descriptor file\n");
        return 2;
    }
    fclose(f);
    for (unsigned long long k = 0; k < hdr[1]; ++k) {
        long long off;
        memcpy(&off, (unsigned char *)&d + rel[k], 8);
        void *p = off < 0 ? NULL : (void *)(blk + off);
        memcpy((unsigned char *)&d + rel[k], &p, sizeof p);
    }

    /* an invalid call first: the error convention (status + message) */
    qgpu_handle *h = NULL;
    if (qgpu_create(NULL, 1, &h) == QGPU_OK) { fprintf(stderr, "null descriptor accepted\n"); return 1; }

    if (qgpu_create(&d, 1, &h) != QGPU_OK) return fail("qgpu_create");
    if (qgpu_build_lists(h) != QGPU_OK) return fail("qgpu_build_lists");
    const int n3 = 3 * d.natom;
    double *grad = calloc((size_t)n3, sizeof(double));
    qgpu_energies E;
    qgpu_qenergy EQ[QGPU_MAX_STATES];
    if (qgpu_forces(h, 0, QGPU_TERMS_ALL, grad, &E, EQ) != QGPU_OK) return fail("qgpu_forces");
    const char *names[12] = {"QEL", "QVdW", "EL", "VdW", "QBND", "QANG", "QTOR", "QIMP", "BND", "ANG", "TOR", "IMP"};
    const double got[12] = {EQ[0].qp_el + EQ[0].qw_el, EQ[0].qp_vdw + EQ[0].qw_vdw,
                            E.pp_el + E.pw_el + E.ww_el, E.pp_vdw + E.pw_vdw + E.ww_vdw,
                            EQ[0].q_bond, EQ[0].q_angle, EQ[0].q_torsion, EQ[0].q_improper,
                            E.p_bond, E.p_angle, E.p_torsion, E.p_improper};
    int bad = 0;
    for (int c = 0; c < 12; ++c) {
        const double want = atof(argv[3 + c]);
        const int ok = fabs(round(got[c] * 100.0) / 100.0 - want) < 1e-9;
        printf("%-5s %12.4f  printed %10.2f  %s\n", names[c], got[c], want, ok ? "ok" : "DIFFERS");
        bad |= !ok;
    }
    double gmax = 0.0;
    for (int k = 0; k < n3; ++k) gmax = fmax(gmax, fabs(grad[k]));
    if (!(gmax > 0.0 && gmax < 1e4)) { printf("gradient out of range: %g\n", gmax); bad = 1; }

    /* SHAKE: displace every atom of the start coordinates (xx) and let
       qgpu_shake restore the constraints, as md_run does after the update */
    double *xx = malloc(sizeof(double) * (size_t)n3), *x = malloc(sizeof(double) * (size_t)n3);
    memcpy(xx, d.x, sizeof(double) * (size_t)n3);
    for (int k = 0; k < n3; ++k) x[k] = xx[k] + 0.004 * sin(0.37 * k + 1.0);
    double before = 0.0, worst = 0.0;
    int ncon = 0;
    for (int m = 0; m < d.shake_molecules; ++m)
        for (int c = d.shake_first[m]; c < d.shake_first[m + 1]; ++c) {
            const int i = d.shake_i[c], j = d.shake_j[c];
            const double dx = x[3 * i] - x[3 * j], dy = x[3 * i + 1] - x[3 * j + 1], dz = x[3 * i + 2] - x[3 * j + 2];
            before = fmax(before, fabs(dx * dx + dy * dy + dz * dz - d.shake_dist2[c]) / d.shake_dist2[c]);
        }
    int32_t niter = 0;
    if (qgpu_shake(h, 0, xx, x, &niter) != QGPU_OK) return fail("qgpu_shake");
    for (int m = 0; m < d.shake_molecules; ++m)
        for (int c = d.shake_first[m]; c < d.shake_first[m + 1]; ++c, ++ncon) {
            const int i = d.shake_i[c], j = d.shake_j[c];
            const double dx = x[3 * i] - x[3 * j], dy = x[3 * i + 1] - x[3 * j + 1], dz = x[3 * i + 2] - x[3 * j + 2];
            worst = fmax(worst, fabs(dx * dx + dy * dy + dz * dz - d.shake_dist2[c]) / d.shake_dist2[c]);
        }
    printf("shake: %d constraints, %d iterations per molecule, worst |r^2 - d0^2|/d0^2 %.3g before, %.3g after\n",
           ncon, niter, before, worst);
    if (!(ncon > 0 && niter >= 1 && worst < 0.5 * before)) bad = 1;
    FILE *fo = fopen(argv[2], "wb");
    if (!fo || fwrite(x, sizeof(double), (size_t)n3, fo) != (size_t)n3) { fprintf(stderr, "cannot write %s\n", argv[2]); return 2; }
    fclose(fo);

    if (qgpu_destroy(h) != QGPU_OK) return fail("qgpu_destroy");
    free(grad); free(xx); free(x); free(rel); free(blk);
    printf(bad ? "FAILED\n" : "all checks passed\n");
    return bad;
}
