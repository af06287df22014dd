/*
 * phgpu_io.h -- PHASTA's POSIX file format (phastaIO) and the mesh/restart
 * reads and writes of the compressible solver, as a C ABI on the host.
 *
 * The entry points replace, with the same argument meaning, these reference
 * routines (paths within the PHASTA project):
 *
 *   phgpu_io_openfile        openfile        phastaIO/phastaIO.cc:916-1109 (POSIX branch)
 *   phgpu_io_closefile       closefile       phastaIO/phastaIO.cc:1120-1263 (POSIX branch)
 *   phgpu_io_readheader      readheader      phastaIO/phastaIO.cc:1271-1448, readHeader :197-306
 *   phgpu_io_readdatablock   readdatablock   phastaIO/phastaIO.cc:1483-1622, readDataBlock :1450-1481
 *   phgpu_io_writeheader     writeheader     phastaIO/phastaIO.cc:1646-1817, writeHeader :1624-1644
 *   phgpu_io_writedatablock  writedatablock  phastaIO/phastaIO.cc:1852-1996, writeDataBlock :1819-1850
 *   phgpu_io_writestring     writestring     phastaIO/phastaIO.cc:2011-2017
 *   phgpu_io_togglestrictmode togglestrictmode phastaIO/phastaIO.cc:2042
 *   phgpu_io_write_restart   restar('out ') + Write_Restart
 *                            phSolver/common/restar.f:53-80, phSolver/common/new_interface.c:240-330
 *   phgpu_io_read_restart    the restart part of readnblk + restar('in  ')
 *                            phSolver/common/readnblk.f:480-545, restar.f:34-49
 *   phgpu_io_geombc_open ... the geombc part of readnblk with genblkPosix and genbkbPosix
 *                            phSolver/common/readnblk.f:112-385, genblkPosix.f:1-111,
 *                            genbkbPosix.f:1-179 (single rank: no ilwork)
 *   phgpu_io_genibc          geniBC          phSolver/common/genibc.f:1-56
 *   phgpu_io_genbc           genBC's conversion of BCinp and genBC1
 *                            phSolver/common/genbc.f:48-57, genbc1.f:1-230
 *   phgpu_io_checkphasta     checkphasta's comparison of two case directories
 *                            checkphasta/checkphasta.cpp:26-136 (POSIX files)
 *
 * File names follow the POSIX naming of the reference (phio_posix.cc:26-30,
 * 98-106): "<dir>/geombc.dat.<rank+1>", "<dir>/restart.<step>.<rank+1>".
 * Arrays keep the reference layouts (Fortran column-major, node index fastest;
 * connectivity 1-based as in the files).  Every entry point returns a status
 * from phgpu.h; the message of the last failure of the calling thread is
 * available from phgpu_io_last_error().  Where the reference only prints a
 * warning (a key that is not found, a data block that does not follow its
 * header) the entry points behave as the reference does and report it in the
 * status: PHGPU_ERR_NOTFOUND leaves the outputs untouched.
 */
#ifndef PHGPU_IO_H
#define PHGPU_IO_H

#include "phgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- phastaIO POSIX format ---------------------------------------------- */

/* mode "read", "write" or "append"; *fd > 0 on success, 0 when the file cannot be opened */
int phgpu_io_openfile(const char* filename, const char* mode, int* fd);
int phgpu_io_closefile(int fd, const char* mode);
/* Search the header line of keyphrase (case-insensitive, blanks ignored, '?' matches the
 * rest; from the current position to the end of the file, then once from its start) and
 * read its first nitems integers into values.  datatype "integer" or "double" (the type of
 * the data block that follows), iotype "binary" or "ascii". */
int phgpu_io_readheader(int fd, const char* keyphrase, int* values, int nitems,
                        const char* datatype, const char* iotype);
/* Read the nitems values of the block whose header was read last (byte-swapped when the
 * file's byte-order magic number says so). */
int phgpu_io_readdatablock(int fd, const char* keyphrase, void* values, int nitems,
                           const char* datatype, const char* iotype);
/* Header line "keyphrase : < bytes > v1 v2 ... " announcing ndataitems values of datatype. */
int phgpu_io_writeheader(int fd, const char* keyphrase, const int* values, int nitems,
                         int ndataitems, const char* datatype, const char* iotype);
int phgpu_io_writedatablock(int fd, const char* keyphrase, const void* values, int nitems,
                            const char* datatype, const char* iotype);
int phgpu_io_writestring(int fd, const char* text);
/* strict mode turns the reference's consistency warnings into PHGPU_ERR_IO; returns the new mode */
int phgpu_io_togglestrictmode(void);
const char* phgpu_io_last_error(void);

/* ---- restart files -------------------------------------------------------- */

/* restart.<stepno>.<rank+1> with the byte-order magic number, "solution" and
 * "time derivative of solution" (nshg, ndof, stepno); y and ac (nshg, ndof) in the
 * solver's (u, v, w, p, T, ...) order, written in the file's (p, u, v, w, T, ...) order. */
int phgpu_io_write_restart(const char* dir, int rank, int stepno, int nshg, int ndof,
                           const double* y, const double* ac);
/* Read restart.<irstart>.<rank+1> into y and ac (nshg, ndof), solver order.  A missing
 * "solution" gives y = 0 with p = T = 1, a missing time derivative ac = 0 (readnblk.f:517-523,
 * 552-558).  *lstep receives the step number of the last header read (0 if none). */
int phgpu_io_read_restart(const char* dir, int rank, int irstart, int nshg, int ndof,
                          double* y, double* ac, int* lstep);

/* ---- geombc files --------------------------------------------------------- */

typedef struct {
    int numnp, nshg, numel, numelb, nen, nelblk, nelblb, numpbc, ntopsh;
    int nsd;              /* second header integer of "co-ordinates" */
    int nbccols;          /* columns of "boundary condition array" (size / numpbc) */
} phgpu_geombc_info;

typedef struct {
    int neltp, nenl, ipordl, nshl, nshlb, nenbl, lcsyst, numnbc;  /* nshlb..numnbc: boundary blocks */
} phgpu_topblock;

typedef struct phgpu_geombc phgpu_geombc;

/* Read <dir>/geombc.dat.<rank+1> in readnblk's order; ndof = 5 for the compressible solver. */
int phgpu_io_geombc_open(const char* dir, int rank, int ndof, phgpu_geombc** out);
int phgpu_io_geombc_free(phgpu_geombc* g);
int phgpu_io_geombc_info(const phgpu_geombc* g, phgpu_geombc_info* info);
/* x (numnp, nsd); nBC, iper (nshg); iBCtmp (numpbc); BCinp (numpbc, nbccols), as in the file */
int phgpu_io_geombc_arrays(const phgpu_geombc* g, double* x, int* nBC, int* iBCtmp, double* BCinp,
                           int* iper);
/* interior block iblk (0-based): its header and ien (neltp, nshl) */
int phgpu_io_geombc_interior(const phgpu_geombc* g, int iblk, phgpu_topblock* blk, int* ien);
/* boundary block iblk: ienb (neltp, nshl), iBCB (neltp, 2), BCB (neltp, nshlb, ndof + 1) after
 * genbkbPosix's masking by the flux codes and gensvb's copy to the face nodes */
int phgpu_io_geombc_boundary(const phgpu_geombc* g, int iblk, phgpu_topblock* blk, int* ienb,
                             int* iBCB, double* BCB);

/* iBC(nshg) = iBCtmp(nBC(n)) where nBC(n) != 0, else 0 */
int phgpu_io_genibc(int nshg, int numpbc, const int* nBC, const int* iBCtmp, int* iBC);
/* BC (nshg, ndof + 1) from BCinp (numpbc, ldbc >= ndof + 7) and iBC: genBC's gather by nBC and
 * genBC1's reduction of the velocity constraints.  The surface-normal and slip-wall paths of
 * genBC (genwnm, genotwn, slpwBC) are not part of it: PHGPU_ERR_UNSUPPORTED when a periodic
 * rotation angle (BCinp(:,12)) is non-zero. */
int phgpu_io_genbc(int nshg, int numpbc, int ndof, const int* nBC, const double* BCinp, int ldbc,
                   const int* iBC, double* BC);

/* ---- checkphasta ---------------------------------------------------------- */

/* Largest |difference| of the "solution" fields of restart.<step>.<rank+1> over the time
 * steps present in both directories (ranks 0..nparts-1); *nsteps = number of common steps.
 * The caller compares *maxdiff with its tolerance as checkphasta's exit status does. */
int phgpu_io_checkphasta(const char* left, const char* right, int nparts, double* maxdiff,
                         int* nsteps);

#ifdef __cplusplus
}
#endif

#endif
