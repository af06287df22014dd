/* Prints the size and every field offset of the structs of include/phgpu.h as JSON, so that the
 * ctypes declarations (phasta_gb300/_lib.py) are checked against what a C compiler makes of the
 * header.  Built and run by tests/test_abi.py with gcc; needs no GPU and no library. */
#include <stddef.h>
#include <stdio.h>

#include "../../include/phgpu.h"

#define F(T, f) printf("%s\"%s\": %zu", first++ ? ", " : "", #f, offsetof(T, f))

int main(void) {
    int first;
    printf("{\"phgpu_config\": {\"__size\": %zu, ", sizeof(phgpu_config));
    first = 0;
    F(phgpu_config, Rgas); F(phgpu_config, gamma); F(phgpu_config, gamma1); F(phgpu_config, pr); F(phgpu_config, rmu);
    F(phgpu_config, Dtgl); F(phgpu_config, almi); F(phgpu_config, alfi); F(phgpu_config, gami);
    F(phgpu_config, dtsfct); F(phgpu_config, taucfct); F(phgpu_config, temper); F(phgpu_config, itau);
    F(phgpu_config, ivart); F(phgpu_config, iremoveStabTimeTerm); F(phgpu_config, Navier); F(phgpu_config, ipord);
    F(phgpu_config, EntropyPressure); F(phgpu_config, Kspace); F(phgpu_config, nGMRES); F(phgpu_config, minIters);
    F(phgpu_config, etol); F(phgpu_config, epsM); F(phgpu_config, eGMRES); F(phgpu_config, iter);
    F(phgpu_config, istep); F(phgpu_config, precision); F(phgpu_config, ap_mode); F(phgpu_config, outer_residual);
    F(phgpu_config, idiff); F(phgpu_config, no_graph); F(phgpu_config, iDC); F(phgpu_config, no_pipe);
    F(phgpu_config, precond);
    printf("}, \"phgpu_mesh\": {\"__size\": %zu, ", sizeof(phgpu_mesh));
    first = 0;
    F(phgpu_mesh, nshg); F(phgpu_mesh, nelem); F(phgpu_mesh, ien); F(phgpu_mesh, x); F(phgpu_mesh, nbelem);
    F(phgpu_mesh, ienb); F(phgpu_mesh, iBCB); F(phgpu_mesh, BCB); F(phgpu_mesh, iBC); F(phgpu_mesh, BC);
    F(phgpu_mesh, iper); F(phgpu_mesh, nhex); F(phgpu_mesh, ienh); F(phgpu_mesh, nwedge); F(phgpu_mesh, ienw);
    F(phgpu_mesh, nbblk); F(phgpu_mesh, bblk);
    printf("}, \"phgpu_bnd_block\": {\"__size\": %zu, ", sizeof(phgpu_bnd_block));
    first = 0;
    F(phgpu_bnd_block, lcsyst); F(phgpu_bnd_block, nelem); F(phgpu_bnd_block, ien); F(phgpu_bnd_block, iBCB);
    F(phgpu_bnd_block, BCB);
    printf("}, \"phgpu_stats\": {\"__size\": %zu, ", sizeof(phgpu_stats));
    first = 0;
    F(phgpu_stats, iKs); F(phgpu_stats, lGMRES); F(phgpu_stats, ntotGM); F(phgpu_stats, status);
    F(phgpu_stats, unorm0); F(phgpu_stats, echeck); F(phgpu_stats, eGMRES); F(phgpu_stats, totres);
    F(phgpu_stats, rnorm); F(phgpu_stats, t_assembly_ms); F(phgpu_stats, t_gmres_ms); F(phgpu_stats, net_its);
    F(phgpu_stats, net_fallback);
    printf("}, \"phgpu_net_train_config\": {\"__size\": %zu, ", sizeof(phgpu_net_train_config));
    first = 0;
    F(phgpu_net_train_config, epochs); F(phgpu_net_train_config, npairs); F(phgpu_net_train_config, lr);
    F(phgpu_net_train_config, beta1); F(phgpu_net_train_config, beta2); F(phgpu_net_train_config, eps);
    F(phgpu_net_train_config, clip); F(phgpu_net_train_config, seed); F(phgpu_net_train_config, renormalize);
    printf("}, \"phgpu_net_train_stats\": {\"__size\": %zu, ", sizeof(phgpu_net_train_stats));
    first = 0;
    F(phgpu_net_train_stats, loss_first); F(phgpu_net_train_stats, loss_last); F(phgpu_net_train_stats, ms);
    F(phgpu_net_train_stats, steps);
    printf("}, \"constants\": {\"PHGPU_NET_NPARAM\": %d, \"PHGPU_NET_NTRAIN\": %d, "
           "\"PHGPU_RSTAT_NOALLOC_MAX_N\": %d, \"PHGPU_PRECOND_LEARNED\": %d, \"PHGPU_NET_PLAIN\": %d}}\n",
           PHGPU_NET_NPARAM, PHGPU_NET_NTRAIN, PHGPU_RSTAT_NOALLOC_MAX_N, PHGPU_PRECOND_LEARNED, PHGPU_NET_PLAIN);
    return 0;
}
