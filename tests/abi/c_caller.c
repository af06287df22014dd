/* A plain C caller of the drop-in boundary: reads a mesh, a state and the COMMON values from a
 * binary file, calls phgpu_create, phgpu_elmmfg (ElmMFG) and phgpu_solmfg (SolMFG) through
 * include/phgpu.h, and writes res, rmes, BDiag (ElmMFG) and res, BDiag, Dy (SolMFG) to a second
 * file.  tests/test_gpu_c_caller.py builds it with gcc, feeds it and compares its outputs with
 * the same calls made through the ctypes binding.
 *
 * Input file (little-endian): int32 nshg, nelem, nbelem; int32 ien[4 nelem]; float64 x[3 nshg];
 * int32 iBC[nshg]; float64 BC[6 nshg]; int32 iper[nshg]; int32 ienb[4 nbelem]; int32 iBCB[2 nbelem];
 * float64 BCB[18 nbelem]; float64 y[5 nshg], ac[5 nshg]; then the phgpu_config values in header
 * order: 12 float64 (Rgas .. temper), 9 int32 (itau .. minIters), 3 float64 (etol, epsM, eGMRES),
 * 9 int32 (iter .. no_pipe), int32 precond. */
#include <stdio.h>
#include <stdlib.h>

#include "../../include/phgpu.h"

static void rd(FILE* f, void* p, size_t sz, size_t n) {
    if (fread(p, sz, n, f) != n) {
        fprintf(stderr, "short read\n");
        exit(2);
    }
}

int main(int argc, char** argv) {
    if (argc != 3) {
        fprintf(stderr, "usage: c_caller in.bin out.bin\n");
        return 2;
    }
    FILE* f = fopen(argv[1], "rb");
    if (!f) return 2;
    int nshg, nelem, nb;
    rd(f, &nshg, 4, 1);
    rd(f, &nelem, 4, 1);
    rd(f, &nb, 4, 1);
    int* ien = malloc(sizeof(int) * 4 * (size_t)nelem);
    double* x = malloc(sizeof(double) * 3 * (size_t)nshg);
    int* iBC = malloc(sizeof(int) * (size_t)nshg);
    double* BC = malloc(sizeof(double) * 6 * (size_t)nshg);
    int* iper = malloc(sizeof(int) * (size_t)nshg);
    int* ienb = malloc(sizeof(int) * 4 * (size_t)(nb + 1));
    int* iBCB = malloc(sizeof(int) * 2 * (size_t)(nb + 1));
    double* BCB = malloc(sizeof(double) * 18 * (size_t)(nb + 1));
    double* y = malloc(sizeof(double) * 5 * (size_t)nshg);
    double* ac = malloc(sizeof(double) * 5 * (size_t)nshg);
    rd(f, ien, 4, 4 * (size_t)nelem);
    rd(f, x, 8, 3 * (size_t)nshg);
    rd(f, iBC, 4, (size_t)nshg);
    rd(f, BC, 8, 6 * (size_t)nshg);
    rd(f, iper, 4, (size_t)nshg);
    rd(f, ienb, 4, 4 * (size_t)nb);
    rd(f, iBCB, 4, 2 * (size_t)nb);
    rd(f, BCB, 8, 18 * (size_t)nb);
    rd(f, y, 8, 5 * (size_t)nshg);
    rd(f, ac, 8, 5 * (size_t)nshg);
    phgpu_config c;
    double d12[12], d3[3];
    int i9[9], j9[9], pc;
    rd(f, d12, 8, 12);
    rd(f, i9, 4, 9);
    rd(f, d3, 8, 3);
    rd(f, j9, 4, 9);
    rd(f, &pc, 4, 1);
    fclose(f);
    c.Rgas = d12[0]; c.gamma = d12[1]; c.gamma1 = d12[2]; c.pr = d12[3]; c.rmu = d12[4];
    c.Dtgl = d12[5]; c.almi = d12[6]; c.alfi = d12[7]; c.gami = d12[8];
    c.dtsfct = d12[9]; c.taucfct = d12[10]; c.temper = d12[11];
    c.itau = i9[0]; c.ivart = i9[1]; c.iremoveStabTimeTerm = i9[2]; c.Navier = i9[3]; c.ipord = i9[4];
    c.EntropyPressure = i9[5]; c.Kspace = i9[6]; c.nGMRES = i9[7]; c.minIters = i9[8];
    c.etol = d3[0]; c.epsM = d3[1]; c.eGMRES = d3[2];
    c.iter = j9[0]; c.istep = j9[1]; c.precision = j9[2]; c.ap_mode = j9[3]; c.outer_residual = j9[4];
    c.idiff = j9[5]; c.no_graph = j9[6]; c.iDC = j9[7]; c.no_pipe = j9[8]; c.precond = pc;
    phgpu_mesh m = {0};
    m.nshg = nshg;
    m.nelem = nelem;
    m.ien = ien;
    m.x = x;
    m.nbelem = nb;
    m.ienb = nb ? ienb : NULL;
    m.iBCB = nb ? iBCB : NULL;
    m.BCB = nb ? BCB : NULL;
    m.iBC = iBC;
    m.BC = BC;
    m.iper = iper;
    phgpu_ctx* ctx = NULL;
    int rc = phgpu_create(&m, &c, &ctx);
    if (rc != PHGPU_OK) {
        fprintf(stderr, "phgpu_create: %d\n", rc);
        return 1;
    }
    const size_t n5 = 5 * (size_t)nshg, n25 = 25 * (size_t)nshg;
    double* res = calloc(n5, sizeof(double));
    double* rmes = calloc(n5, sizeof(double));
    double* bd = calloc(n25, sizeof(double));
    double* res2 = calloc(n5, sizeof(double));
    double* bd2 = calloc(n25, sizeof(double));
    double* Dy = calloc(n5, sizeof(double));
    rc = phgpu_elmmfg(ctx, y, ac, res, rmes, bd, 1);
    if (rc != PHGPU_OK) {
        fprintf(stderr, "phgpu_elmmfg: %d %s\n", rc, phgpu_last_error(ctx));
        return 1;
    }
    phgpu_stats st = {0};
    rc = phgpu_solmfg(ctx, y, ac, res2, bd2, Dy, &st);
    if (rc != PHGPU_OK) {
        fprintf(stderr, "phgpu_solmfg: %d %s\n", rc, phgpu_last_error(ctx));
        return 1;
    }
    FILE* o = fopen(argv[2], "wb");
    if (!o) return 2;
    fwrite(res, 8, n5, o);
    fwrite(rmes, 8, n5, o);
    fwrite(bd, 8, n25, o);
    fwrite(res2, 8, n5, o);
    fwrite(bd2, 8, n25, o);
    fwrite(Dy, 8, n5, o);
    fwrite(&st.iKs, 4, 1, o);
    fclose(o);
    printf("c_caller: ElmMFG and SolMFG ok, %d Krylov iterations\n", st.iKs);
    phgpu_destroy(ctx);
    return 0;
}
