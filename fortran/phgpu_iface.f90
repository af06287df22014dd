! phgpu_iface.f90 -- ISO_C_BINDING interface of include/phgpu.h for a PHASTA
! build (compressible solver): the structs and the bind(C) interfaces of the
! phgpu_* entry points.  The drop-in replacements of the reference routines,
! with their own names and argument lists, are in phgpu_shims.f (they use
! this module).  Compiled only by a Fortran compiler.
module phgpu_iface
  use iso_c_binding
  implicit none

  integer(c_int), parameter :: PHGPU_OK = 0
  integer(c_int), parameter :: PHGPU_FP64 = 0, PHGPU_MIXED = 1
  integer(c_int), parameter :: PHGPU_AP_FD = 0, PHGPU_AP_LINEAR = 1, PHGPU_AP_SPARSE = 2, PHGPU_AP_EBE = 3
  integer(c_int), parameter :: PHGPU_RES_FP64 = 0, PHGPU_RES_GALERKIN64 = 1, PHGPU_RES_SPLITDF = 2
  integer(c_int), parameter :: PHGPU_PRECOND_BDIAG = 0, PHGPU_PRECOND_LEARNED = 1

  type, bind(C) :: phgpu_config
     real(c_double) :: Rgas, gamma, gamma1, pr, rmu
     real(c_double) :: Dtgl, almi, alfi, gami
     real(c_double) :: dtsfct, taucfct, temper
     integer(c_int) :: itau, ivart, iremoveStabTimeTerm, Navier, ipord, EntropyPressure
     integer(c_int) :: Kspace, nGMRES, minIters
     real(c_double) :: etol, epsM, eGMRES
     integer(c_int) :: iter, istep
     integer(c_int) :: precision, ap_mode, outer_residual
     integer(c_int) :: idiff         ! 0 or 1 (global diffusive-flux reconstruction)
     integer(c_int) :: no_graph, iDC, no_pipe, precond
  end type

  ! a block of boundary hexes (lcsyst 2) or wedges (3: triangle face, 4: quadrilateral face)
  type, bind(C) :: phgpu_bnd_block
     integer(c_int) :: lcsyst, nelem
     type(c_ptr)    :: ien, iBCB, BCB
  end type

  type, bind(C) :: phgpu_mesh
     integer(c_int) :: nshg, nelem
     type(c_ptr)    :: ien, x
     integer(c_int) :: nbelem
     type(c_ptr)    :: ienb, iBCB, BCB, iBC, BC, iper
     integer(c_int) :: nhex          ! blocks with lcsyst 2 (mien(iblk)%p of nshl = 8)
     type(c_ptr)    :: ienh
     integer(c_int) :: nwedge        ! blocks with lcsyst 3 (nshl = 6)
     type(c_ptr)    :: ienw
     integer(c_int) :: nbblk         ! boundary hex and wedge blocks
     type(c_ptr)    :: bblk          ! nbblk phgpu_bnd_block
  end type

  type, bind(C) :: phgpu_stats
     integer(c_int) :: iKs, lGMRES, ntotGM, status
     real(c_double) :: unorm0, echeck, eGMRES, totres, rnorm, t_assembly_ms, t_gmres_ms
     integer(c_int) :: net_its, net_fallback
  end type

  interface
     integer(c_int) function phgpu_create(mesh, cfg, ctx) bind(C, name="phgpu_create")
       import :: c_int, c_ptr, phgpu_mesh, phgpu_config
       type(phgpu_mesh), intent(in) :: mesh
       type(phgpu_config), intent(in) :: cfg
       type(c_ptr), intent(out) :: ctx
     end function
     integer(c_int) function phgpu_set_config(ctx, cfg) bind(C, name="phgpu_set_config")
       import :: c_int, c_ptr, phgpu_config
       type(c_ptr), value :: ctx
       type(phgpu_config), intent(in) :: cfg
     end function
     integer(c_int) function phgpu_destroy(ctx) bind(C, name="phgpu_destroy")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function
     integer(c_int) function phgpu_set_bc(ctx, BC) bind(C, name="phgpu_set_bc")
       import :: c_int, c_double, c_ptr
       type(c_ptr), value :: ctx
       real(c_double), intent(in) :: BC(*)
     end function
     integer(c_int) function phgpu_net_set_weights(ctx, w, n) bind(C, name="phgpu_net_set_weights")
       import :: c_int, c_float, c_ptr
       type(c_ptr), value :: ctx
       real(c_float), intent(in) :: w(*)
       integer(c_int), value :: n
     end function
     integer(c_int) function phgpu_elmmfg(ctx, y, ac, res, rmes, bdiag, iprec) bind(C, name="phgpu_elmmfg")
       import :: c_int, c_double, c_ptr
       type(c_ptr), value :: ctx
       real(c_double), intent(in) :: y(*), ac(*)
       real(c_double), intent(out) :: res(*), rmes(*), bdiag(*)
       integer(c_int), value :: iprec
     end function
     integer(c_int) function phgpu_itrres(ctx, yp, yc, ac, rmes) bind(C, name="phgpu_itrres")
       import :: c_int, c_double, c_ptr
       type(c_ptr), value :: ctx
       real(c_double), intent(in) :: yp(*), yc(*), ac(*)
       real(c_double), intent(inout) :: rmes(*)
     end function
     integer(c_int) function phgpu_solmfg(ctx, y, ac, res, bdiag, Dy, st) bind(C, name="phgpu_solmfg")
       import :: c_int, c_double, c_ptr, phgpu_stats
       type(c_ptr), value :: ctx
       real(c_double), intent(in) :: y(*), ac(*)
       real(c_double), intent(out) :: res(*), bdiag(*), Dy(*)
       type(phgpu_stats), intent(inout) :: st
     end function
     integer(c_int) function phgpu_time_step(ctx, yold, acold, y, ac, nitr, st) bind(C, name="phgpu_time_step")
       import :: c_int, c_double, c_ptr, phgpu_stats
       type(c_ptr), value :: ctx
       real(c_double), intent(inout) :: yold(*), acold(*)
       real(c_double), intent(out) :: y(*), ac(*)
       integer(c_int), value :: nitr
       type(phgpu_stats), intent(inout) :: st
     end function
     integer(c_int) function phgpu_genadj(mesh, nnz, colm, rowp, icnt) bind(C, name="phgpu_genadj")
       import :: c_int, phgpu_mesh
       type(phgpu_mesh), intent(in) :: mesh
       integer(c_int), value :: nnz
       integer(c_int), intent(out) :: colm(*), rowp(*), icnt
     end function
     integer(c_int) function phgpu_elmgmrs(ctx, y, ac, res, bdiag, lhsK) bind(C, name="phgpu_elmgmrs")
       import :: c_int, c_double, c_ptr
       type(c_ptr), value :: ctx
       real(c_double), intent(in) :: y(*), ac(*)
       real(c_double), intent(out) :: res(*), bdiag(*), lhsK(*)
     end function
     integer(c_int) function phgpu_spsi3pre(ctx, bdiag, lhsK) bind(C, name="phgpu_spsi3pre")
       import :: c_int, c_double, c_ptr
       type(c_ptr), value :: ctx
       real(c_double), intent(in) :: bdiag(*)
       real(c_double), intent(inout) :: lhsK(*)
     end function
     integer(c_int) function phgpu_sparseap(ctx, lhsK, p) bind(C, name="phgpu_sparseap")
       import :: c_int, c_double, c_ptr
       type(c_ptr), value :: ctx
       real(c_double), intent(in) :: lhsK(*)
       real(c_double), intent(inout) :: p(*)
     end function
     integer(c_int) function phgpu_solgmrs(ctx, y, ac, lhs, res, bdiag, Dy, lhsK, st) bind(C, name="phgpu_solgmrs")
       import :: c_int, c_double, c_ptr, phgpu_stats
       type(c_ptr), value :: ctx
       real(c_double), intent(in) :: y(*), ac(*)
       integer(c_int), value :: lhs
       real(c_double), intent(out) :: res(*), bdiag(*), Dy(*), lhsK(*)
       type(phgpu_stats), intent(inout) :: st
     end function
     integer(c_int) function phgpu_elmgmre(ctx, y, ac, res, bdiag, EGmass) bind(C, name="phgpu_elmgmre")
       import :: c_int, c_double, c_ptr
       type(c_ptr), value :: ctx
       real(c_double), intent(in) :: y(*), ac(*)
       real(c_double), intent(out) :: res(*), bdiag(*), EGmass(*)
     end function
     integer(c_int) function phgpu_i3pre(ctx, bdiag, EGmass) bind(C, name="phgpu_i3pre")
       import :: c_int, c_double, c_ptr
       type(c_ptr), value :: ctx
       real(c_double), intent(in) :: bdiag(*)
       real(c_double), intent(inout) :: EGmass(*)
     end function
     integer(c_int) function phgpu_au1gmr(ctx, EGmass, p) bind(C, name="phgpu_au1gmr")
       import :: c_int, c_double, c_ptr
       type(c_ptr), value :: ctx
       real(c_double), intent(in) :: EGmass(*)
       real(c_double), intent(inout) :: p(*)
     end function
     integer(c_int) function phgpu_solgmre(ctx, y, ac, res, bdiag, Dy, EGmass, st) bind(C, name="phgpu_solgmre")
       import :: c_int, c_double, c_ptr, phgpu_stats
       type(c_ptr), value :: ctx
       real(c_double), intent(in) :: y(*), ac(*)
       real(c_double), intent(out) :: res(*), bdiag(*), Dy(*), EGmass(*)
       type(phgpu_stats), intent(inout) :: st
     end function
     type(c_ptr) function phgpu_last_error(ctx) bind(C, name="phgpu_last_error")
       import :: c_ptr
       type(c_ptr), value :: ctx
     end function
     ! include/phgpu_io.h: PHASTA files (strings are NUL-terminated: c_char_'...'//c_null_char)
     integer(c_int) function phgpu_io_openfile(filename, mode, fd) bind(C, name="phgpu_io_openfile")
       import :: c_int, c_char
       character(kind=c_char), intent(in) :: filename(*), mode(*)
       integer(c_int), intent(out) :: fd
     end function
     integer(c_int) function phgpu_io_closefile(fd, mode) bind(C, name="phgpu_io_closefile")
       import :: c_int, c_char
       integer(c_int), value :: fd
       character(kind=c_char), intent(in) :: mode(*)
     end function
     integer(c_int) function phgpu_io_readheader(fd, key, values, nitems, datatype, iotype) &
         bind(C, name="phgpu_io_readheader")
       import :: c_int, c_char
       integer(c_int), value :: fd, nitems
       character(kind=c_char), intent(in) :: key(*), datatype(*), iotype(*)
       integer(c_int), intent(inout) :: values(*)
     end function
     integer(c_int) function phgpu_io_readdatablock(fd, key, values, nitems, datatype, iotype) &
         bind(C, name="phgpu_io_readdatablock")
       import :: c_int, c_char, c_ptr
       integer(c_int), value :: fd, nitems
       character(kind=c_char), intent(in) :: key(*), datatype(*), iotype(*)
       type(c_ptr), value :: values
     end function
     integer(c_int) function phgpu_io_writeheader(fd, key, values, nitems, ndata, datatype, iotype) &
         bind(C, name="phgpu_io_writeheader")
       import :: c_int, c_char
       integer(c_int), value :: fd, nitems, ndata
       character(kind=c_char), intent(in) :: key(*), datatype(*), iotype(*)
       integer(c_int), intent(in) :: values(*)
     end function
     integer(c_int) function phgpu_io_writedatablock(fd, key, values, nitems, datatype, iotype) &
         bind(C, name="phgpu_io_writedatablock")
       import :: c_int, c_char, c_ptr
       integer(c_int), value :: fd, nitems
       character(kind=c_char), intent(in) :: key(*), datatype(*), iotype(*)
       type(c_ptr), value :: values
     end function
     integer(c_int) function phgpu_io_write_restart(dir, rank, stepno, nshg, ndof, y, ac) &
         bind(C, name="phgpu_io_write_restart")
       import :: c_int, c_char, c_double
       character(kind=c_char), intent(in) :: dir(*)
       integer(c_int), value :: rank, stepno, nshg, ndof
       real(c_double), intent(in) :: y(*), ac(*)
     end function
     integer(c_int) function phgpu_io_read_restart(dir, rank, irstart, nshg, ndof, y, ac, lstep) &
         bind(C, name="phgpu_io_read_restart")
       import :: c_int, c_char, c_double
       character(kind=c_char), intent(in) :: dir(*)
       integer(c_int), value :: rank, irstart, nshg, ndof
       real(c_double), intent(out) :: y(*), ac(*)
       integer(c_int), intent(out) :: lstep
     end function
     integer(c_int) function phgpu_io_genibc(nshg, numpbc, nBC, iBCtmp, iBC) bind(C, name="phgpu_io_genibc")
       import :: c_int
       integer(c_int), value :: nshg, numpbc
       integer(c_int), intent(in) :: nBC(*), iBCtmp(*)
       integer(c_int), intent(out) :: iBC(*)
     end function
     integer(c_int) function phgpu_io_genbc(nshg, numpbc, ndof, nBC, BCinp, ldbc, iBC, BC) &
         bind(C, name="phgpu_io_genbc")
       import :: c_int, c_double
       integer(c_int), value :: nshg, numpbc, ndof, ldbc
       integer(c_int), intent(in) :: nBC(*), iBC(*)
       real(c_double), intent(in) :: BCinp(*)
       real(c_double), intent(out) :: BC(*)
     end function
  end interface

  type(c_ptr), save :: phgpu_ctx = c_null_ptr
end module phgpu_iface
