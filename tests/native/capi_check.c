/*
 * A C caller of libchimes_gb300.so that sees nothing but include/chimes_gb300.h:
 * the design matrix of an fm_setup.in's trajectory (cg_assemble, FP64) and the MD
 * forces of one configuration with given coefficients (cg_md_force), written as raw
 * little-endian doubles for the test to compare with the reference's fixtures.
 *
 *   capi_check FM_SETUP OUT_A [MD_FM_SETUP MD_FRAME MD_COEF OUT_F]
 *
 * MD_FRAME: int32 natoms, int32 types[natoms], double xyz[3 natoms], double cell[9];
 * MD_COEF: int32 n, double x[n].  OUT_A: int64 rows, int64 cols, then rows x cols
 * doubles; OUT_F: 3 natoms forces then the 11 per-frame scalars.
 */
#include <stdio.h>
#include <stdlib.h>

#include "chimes_gb300.h"

static int fail(const char* what, int rc) {
    fprintf(stderr, "%s failed (status %d): %s\n", what, rc, cg_last_error());
    return 1;
}

static void* slurp(const char* path, size_t* n) {
    FILE* f = fopen(path, "rb");
    if (!f) return NULL;
    fseek(f, 0, SEEK_END);
    long len = ftell(f);
    fseek(f, 0, SEEK_SET);
    void* p = malloc(len > 0 ? (size_t)len : 1);
    if (p && fread(p, 1, (size_t)len, f) != (size_t)len) { free(p); p = NULL; }
    fclose(f);
    *n = (size_t)len;
    return p;
}

int main(int argc, char** argv) {
    if (argc != 3 && argc != 7) {
        fprintf(stderr, "usage: capi_check FM_SETUP OUT_A [MD_FM_SETUP MD_FRAME MD_COEF OUT_F]\n");
        return 2;
    }
    cg_model* m = NULL;
    cg_frames* fr = NULL;
    cg_session* s = NULL;
    int rc = cg_model_load(argv[1], &m);
    if (rc) return fail("cg_model_load", rc);
    if ((rc = cg_frames_read(m, NULL, 0, &fr))) return fail("cg_frames_read", rc);
    if ((rc = cg_session_create(m, 0, &s))) return fail("cg_session_create", rc);
    int ncols = 0;
    int64_t rows = 0;
    if ((rc = cg_model_columns(m, NULL, NULL, NULL, NULL, &ncols))) return fail("cg_model_columns", rc);
    if ((rc = cg_frames_rows(fr, &rows, NULL))) return fail("cg_frames_rows", rc);
    double* A = (double*)malloc(sizeof(double) * (size_t)rows * ncols);
    if (!A) return 3;
    if ((rc = cg_assemble(s, fr, CG_FP64, A, ncols))) return fail("cg_assemble", rc);
    FILE* out = fopen(argv[2], "wb");
    if (!out) return 3;
    int64_t hdr[2] = {rows, ncols};
    fwrite(hdr, sizeof(hdr), 1, out);
    fwrite(A, sizeof(double), (size_t)rows * ncols, out);
    fclose(out);
    free(A);
    cg_frames_free(fr);
    cg_session_free(s);
    cg_model_free(m);
    if (argc == 3) return 0;

    /* MD forces */
    size_t nb = 0, nc = 0;
    char* frame = (char*)slurp(argv[4], &nb);
    char* coef = (char*)slurp(argv[5], &nc);
    if (!frame || !coef || nb < 4 || nc < 4) return 3;
    const int natoms = *(const int*)frame;
    const int* types = (const int*)(frame + 4);
    const double* xyz = (const double*)(frame + 4 + 4 * (size_t)natoms);
    const double* cell = xyz + 3 * (size_t)natoms;
    const int nx = *(const int*)coef;
    const double* x = (const double*)(coef + 4);
    if ((rc = cg_model_load(argv[3], &m))) return fail("cg_model_load (MD)", rc);
    if ((rc = cg_session_create(m, 0, &s))) return fail("cg_session_create (MD)", rc);
    if ((rc = cg_md_setup(s, x, nx, CG_FP64, CG_MD_ENERGY_OFFSETS, 0.01, 1.0e4))) return fail("cg_md_setup", rc);
    if ((rc = cg_frames_create(m, 1, &natoms, types, xyz, NULL, cell, NULL, NULL, 0, &fr)))
        return fail("cg_frames_create", rc);
    if ((rc = cg_frames_independent(fr))) return fail("cg_frames_independent", rc);
    double* F = (double*)malloc(sizeof(double) * (3 * (size_t)natoms + 11));
    if (!F) return 3;
    if ((rc = cg_md_force(s, fr, F, F + 3 * natoms))) return fail("cg_md_force", rc);
    out = fopen(argv[6], "wb");
    if (!out) return 3;
    fwrite(F, sizeof(double), 3 * (size_t)natoms + 11, out);
    fclose(out);
    free(F);
    free(frame);
    free(coef);
    cg_frames_free(fr);
    cg_session_free(s);
    cg_model_free(m);
    printf("capi_check: A %lld x %d, MD forces of %d atoms\n", (long long)rows, ncols, natoms);
    return 0;
}
