c phgpu_shims.f -- drop-in replacements of PHASTA's compressible hot-path
c routines, with the reference's names and argument lists:
c
c   ElmMFG   phSolver/compressible/elmmfg.f:1-5
c   ItrRes   phSolver/compressible/itrres.f:1-5
c   SolMFG   phSolver/compressible/solmfg.f:1-7
c   ElmGMRs  phSolver/compressible/elmgmr.f:280-285
c   SolGMRs  phSolver/compressible/solgmr.f:368-374
c   ElmGMRe  phSolver/compressible/elmgmr.f:1-5
c   SolGMRe  phSolver/compressible/solgmr.f:1-6
c
c A PHASTA build links this file (and phgpu_iface.f90, libphgpu.so) in
c place of those routines; itrdrv and every other caller stay as they are.
c What the reference reads from COMMON (common.h) and from pointer_data
c (element blocks mien/mienb/miBCB/mBCB, lcblk/lcblkb) is read here the same
c way: the first call creates the GPU context from the element blocks, and
c every call hands the current COMMON values (phgpu_config) and BC to it.
c A non-zero status of the GPU path ends in the reference's error(), as
c the reference's own checks do (common/error.f).
c
c Limits (those of include/phgpu.h): linear tets, hexes and wedges
c (lcsyst 1-3), boundary tets only, constant viscosity (matflg(2) = 0),
c one rank.  rerr (the error indicators of ierrcalc = 1) is not computed.
c
c The precision and the product default to the reference arithmetic (FP64,
c finite-difference Au1MFG); phgpu_shim_options (before the first call)
c selects the mixed-precision forms.
c
        module phgpu_shim_state
        use iso_c_binding
        use phgpu_iface
        implicit none
        type(c_ptr), save :: hctx = c_null_ptr
        integer(c_int), save :: oprec = PHGPU_FP64
        integer(c_int), save :: oap = PHGPU_AP_FD
        integer(c_int), save :: ores = PHGPU_RES_FP64
        integer(c_int), save :: opc = PHGPU_PRECOND_BDIAG
        integer(c_int), allocatable, target, save :: ient(:), ienh(:)
        integer(c_int), allocatable, target, save :: ienw(:), ienb(:)
        integer(c_int), allocatable, target, save :: ibcbc(:)
        real(c_double), allocatable, target, save :: bcbc(:)
c.... boundary hex and wedge blocks: the phgpu_bnd_block list and its arrays
        type(phgpu_bnd_block), allocatable, target, save :: bblks(:)
        integer(c_int), allocatable, target, save :: ienbt(:), ibcbt(:)
        real(c_double), allocatable, target, save :: bcbt(:)
        end module
c
c.... options of the GPU path (call before the first solve)
c
        subroutine phgpu_shim_options (iprecision, iapmode, iouter,
     &                                 iprecond)
        use phgpu_shim_state
        implicit none
        integer iprecision, iapmode, iouter, iprecond
        oprec = iprecision
        oap = iapmode
        ores = iouter
        opc = iprecond
        end
c
c.... the context of this run (created on the first call) with the current
c     COMMON values and BC
c
        subroutine phgpu_shim_setup (x, iBC, BC, iper, ctx)
        use pointer_data
        use phgpu_shim_state
        include "common.h"
        dimension x(numnp,nsd), iBC(nshg), BC(nshg,ndofBC), iper(nshg)
        target x, iBC, BC
        type(c_ptr) ctx
        type(phgpu_mesh) :: m
        type(phgpu_config) :: cfg
        integer(c_int) :: rc
        integer(c_int), allocatable, target :: iperc(:)
        integer nt, nh, nw, nb, ib, i, j, k, ie
        integer nbl, nbt, nbi, nbc, nsl, nsb
c
        if (numpe .gt. 1) call error ('phgpushm', 'numpe   ', numpe)
        if (matflg(2,1) .ne. 0) call error ('phgpushm', 'matflg2 ',
     &                                     matflg(2,1))
c
c.... the phgpu_config of the COMMON values (common.h)
c
        cfg%Rgas = Rgas
        cfg%gamma = gamma
        cfg%gamma1 = gamma1
        cfg%pr = pr
        cfg%rmu = datmat(1,2,1)
        cfg%Dtgl = Dtgl
        cfg%almi = almi
        cfg%alfi = alfi
        cfg%gami = gami
        cfg%dtsfct = dtsfct
        cfg%taucfct = taucfct
        cfg%temper = temper
        cfg%itau = itau
        cfg%ivart = ivart
        cfg%iremoveStabTimeTerm = iremoveStabTimeTerm
        cfg%Navier = navier
        cfg%ipord = ipord
        cfg%EntropyPressure = EntropyPressure
        cfg%Kspace = Kspace
        cfg%nGMRES = nGMRES
        cfg%minIters = minIters
        cfg%etol = epstol(1)
        cfg%epsM = epsM
        cfg%eGMRES = eGMRES
        cfg%iter = iter
        cfg%istep = istep
        cfg%precision = oprec
        cfg%ap_mode = oap
        cfg%outer_residual = ores
        cfg%idiff = idiff
        cfg%no_graph = 0
        cfg%iDC = iDC
        cfg%no_pipe = 0
        cfg%precond = opc
c
        if (.not. c_associated(hctx)) then
c
c.... element blocks as 0-based connectivity, by topology (lcblk(3,:))
c
          nt = 0
          nh = 0
          nw = 0
          do ib = 1, nelblk
            i = lcblk(1,ib+1) - lcblk(1,ib)
            select case (lcblk(3,ib))
            case (1)
              nt = nt + i
            case (2)
              nh = nh + i
            case (3)
              nw = nw + i
            case default
              call error ('phgpushm', 'lcsyst  ', lcblk(3,ib))
            end select
          enddo
          allocate (ient(max(1,4*nt)), ienh(max(1,8*nh)))
          allocate (ienw(max(1,6*nw)))
          nt = 0
          nh = 0
          nw = 0
          do ib = 1, nelblk
            do ie = 1, lcblk(1,ib+1) - lcblk(1,ib)
              select case (lcblk(3,ib))
              case (1)
                do j = 1, 4
                  ient(4*nt+j) = abs(mien(ib)%p(ie,j)) - 1
                enddo
                nt = nt + 1
              case (2)
                do j = 1, 8
                  ienh(8*nh+j) = abs(mien(ib)%p(ie,j)) - 1
                enddo
                nh = nh + 1
              case (3)
                do j = 1, 6
                  ienw(6*nw+j) = abs(mien(ib)%p(ie,j)) - 1
                enddo
                nw = nw + 1
              end select
            enddo
          enddo
c
c.... boundary tets (face first), their iBCB and BCB
c
          nb = 0
          do ib = 1, nelblb
            if (lcblkb(3,ib) .lt. 1 .or. lcblkb(3,ib) .gt. 3)
     &        call error ('phgpushm', 'bndtopo ', lcblkb(3,ib))
            if (lcblkb(3,ib) .eq. 1)
     &        nb = nb + lcblkb(1,ib+1) - lcblkb(1,ib)
          enddo
          allocate (ienb(max(1,4*nb)), ibcbc(max(1,2*nb)))
          allocate (bcbc(max(1,18*nb)))
          bcbc = 0d0
          nb = 0
          do ib = 1, nelblb
            if (lcblkb(3,ib) .ne. 1) cycle
            do ie = 1, lcblkb(1,ib+1) - lcblkb(1,ib)
              do j = 1, 4
                ienb(4*nb+j) = abs(mienb(ib)%p(ie,j)) - 1
              enddo
              ibcbc(2*nb+1) = miBCB(ib)%p(ie,1)
              ibcbc(2*nb+2) = miBCB(ib)%p(ie,2)
              do j = 1, 3
                do k = 1, min(6, ndBCB)
                  bcbc(18*nb + 6*(j-1) + k) = mBCB(ib)%p(ie,j,k)
                enddo
              enddo
              nb = nb + 1
            enddo
          enddo
          m%nshg = nshg
          m%nelem = nt
          m%ien = c_loc(ient)
          m%x = c_loc(x)
          m%nbelem = nb
          m%ienb = c_loc(ienb)
          m%iBCB = c_loc(ibcbc)
          m%BCB = c_loc(bcbc)
          m%iBC = c_loc(iBC)
          m%BC = c_loc(BC)
c.... periodic masters 0-based (phgpu_create copies what it keeps)
          allocate (iperc(nshg))
          do i = 1, nshg
            iperc(i) = iper(i) - 1
          enddo
          m%iper = c_loc(iperc)
          m%nhex = nh
          m%ienh = c_loc(ienh)
          m%nwedge = nw
          m%ienw = c_loc(ienw)
c
c.... boundary hex and wedge blocks, one phgpu_bnd_block each: lcsyst 2
c     for hexes, and for wedges the face's node count nenbl as
c     elmmfg.f:187 turns it into the lcsyst of the boundary rule (3
c     triangle, 4 quadrilateral); nshl = lcblkb(9,:), nshlb = lcblkb(10,:)
c
          nbl = 0
          nbt = 0
          nbi = 0
          nbc = 0
          do ib = 1, nelblb
            if (lcblkb(3,ib) .eq. 1) cycle
            i = lcblkb(1,ib+1) - lcblkb(1,ib)
            nbl = nbl + 1
            nbt = nbt + i*lcblkb(9,ib)
            nbi = nbi + 2*i
            nbc = nbc + 6*i*lcblkb(10,ib)
          enddo
          allocate (bblks(max(1,nbl)), ienbt(max(1,nbt)))
          allocate (ibcbt(max(1,nbi)), bcbt(max(1,nbc)))
          bcbt = 0d0
          nbl = 0
          nbt = 0
          nbi = 0
          nbc = 0
          do ib = 1, nelblb
            if (lcblkb(3,ib) .eq. 1) cycle
            i = lcblkb(1,ib+1) - lcblkb(1,ib)
            nsl = lcblkb(9,ib)
            nsb = lcblkb(10,ib)
            nbl = nbl + 1
            if (lcblkb(3,ib) .eq. 2) then
              bblks(nbl)%lcsyst = 2
            else
              bblks(nbl)%lcsyst = lcblkb(6,ib)
            endif
            bblks(nbl)%nelem = i
            bblks(nbl)%ien = c_loc(ienbt(nbt+1))
            bblks(nbl)%iBCB = c_loc(ibcbt(nbi+1))
            bblks(nbl)%BCB = c_loc(bcbt(nbc+1))
            do ie = 1, i
              do j = 1, nsl
                ienbt(nbt+j) = abs(mienb(ib)%p(ie,j)) - 1
              enddo
              ibcbt(nbi+1) = miBCB(ib)%p(ie,1)
              ibcbt(nbi+2) = miBCB(ib)%p(ie,2)
              do j = 1, nsb
                do k = 1, min(6, ndBCB)
                  bcbt(nbc + 6*(j-1) + k) = mBCB(ib)%p(ie,j,k)
                enddo
              enddo
              nbt = nbt + nsl
              nbi = nbi + 2
              nbc = nbc + 6*nsb
            enddo
          enddo
          m%nbblk = nbl
          m%bblk = c_loc(bblks)
          rc = phgpu_create (m, cfg, hctx)
          deallocate (iperc)
          if (rc .ne. PHGPU_OK) call error ('phgpushm', 'create  ', rc)
        endif
c
        rc = phgpu_set_config (hctx, cfg)
        if (rc .ne. PHGPU_OK) call error ('phgpushm', 'config  ', rc)
        rc = phgpu_set_bc (hctx, BC)
        if (rc .ne. PHGPU_OK) call error ('phgpushm', 'BC      ', rc)
        ctx = hctx
        end
c
c.... the COMMON iteration statistics of a solve (itrpar)
c
        subroutine phgpu_shim_stats (st)
        use phgpu_shim_state
        include "common.h"
        type(phgpu_stats) st
        iKs = st%iKs
        lGMRES = st%lGMRES
        ntotGM = st%ntotGM
        eGMRES = st%eGMRES
        end
c
c----------------------------------------------------------------------
c
        subroutine ElmMFG (y,         ac,        x,
     &                     shp,       shgl,      iBC,
     &                     BC,        shpb,      shglb,
     &                     res,       rmes,      BDiag,
     &                     iper,      ilwork,    rerr)
        use phgpu_shim_state
        include "common.h"
        dimension y(nshg,ndof),         ac(nshg,ndof),
     &            x(numnp,nsd),         iBC(nshg),
     &            BC(nshg,ndofBC),      res(nshg,nflow),
     &            rmes(nshg,nflow),     BDiag(nshg,nflow,nflow),
     &            iper(nshg),           ilwork(nlwork)
        dimension shp(MAXTOP,maxsh,MAXQPT),
     &            shgl(MAXTOP,nsd,maxsh,MAXQPT),
     &            shpb(MAXTOP,maxsh,MAXQPT),
     &            shglb(MAXTOP,nsd,maxsh,MAXQPT)
        real*8  rerr(nshg,10)
        type(c_ptr) ctx
        integer(c_int) :: rc
        call phgpu_shim_setup (x, iBC, BC, iper, ctx)
        rc = phgpu_elmmfg (ctx, y, ac, res, rmes, BDiag, iprec)
        if (rc .ne. PHGPU_OK) call error ('ElmMFG  ', 'phgpu   ', rc)
        end
c
        subroutine ItrRes (yp,        yc,        x,
     &                     shp,       shgl,
     &                     iBC,       BC,        shpb,
     &                     shglb,     rmes,      iper,
     &                     ilwork,    ac)
        use phgpu_shim_state
        include "common.h"
        dimension yp(nshg,ndof),        yc(nshg,ndof),
     &            x(numnp,nsd),         iBC(nshg),
     &            BC(nshg,ndofBC),      rmes(nshg,nflow),
     &            iper(nshg),           ilwork(nlwork),
     &            ac(nshg,ndof)
        dimension shp(MAXTOP,maxsh,MAXQPT),
     &            shgl(MAXTOP,nsd,maxsh,MAXQPT),
     &            shpb(MAXTOP,maxsh,MAXQPT),
     &            shglb(MAXTOP,nsd,maxsh,MAXQPT)
        type(c_ptr) ctx
        integer(c_int) :: rc
        call phgpu_shim_setup (x, iBC, BC, iper, ctx)
        rc = phgpu_itrres (ctx, yp, yc, ac, rmes)
        if (rc .ne. PHGPU_OK) call error ('ItrRes  ', 'phgpu   ', rc)
        end
c
        subroutine SolMFG (y,         ac,        yold,      acold,
     &                     x,
     &                     iBC,       BC,        res,
     &                     BDiag,     HBrg,      eBrg,
     &                     yBrg,      Rcos,      Rsin,      iper,
     &                     ilwork,    shp,       shgl,
     &                     shpb,      shglb,     Dy, rerr)
        use phgpu_shim_state
        include "common.h"
        dimension y(nshg,ndof),         ac(nshg,ndof),
     &            yold(nshg,ndof),      acold(nshg,ndof),
     &            x(numnp,nsd),         iBC(nshg),
     &            BC(nshg,ndofBC),      res(nshg,nflow),
     &            BDiag(nshg,nflow,nflow),
     &            HBrg(Kspace+1,Kspace), eBrg(Kspace+1),
     &            yBrg(Kspace),         Rcos(Kspace),
     &            Rsin(Kspace),         iper(nshg),
     &            ilwork(nlwork),       Dy(nshg,nflow)
        dimension shp(MAXTOP,maxsh,MAXQPT),
     &            shgl(MAXTOP,nsd,maxsh,MAXQPT),
     &            shpb(MAXTOP,maxsh,MAXQPT),
     &            shglb(MAXTOP,nsd,maxsh,MAXQPT)
        real*8  rerr(nshg,10)
        type(c_ptr) ctx
        type(phgpu_stats) :: st
        integer(c_int) :: rc
        call phgpu_shim_setup (x, iBC, BC, iper, ctx)
        st%ntotGM = ntotGM
        rc = phgpu_solmfg (ctx, y, ac, res, BDiag, Dy, st)
        if (rc .ne. PHGPU_OK) call error ('SolMFG  ', 'phgpu   ', rc)
        call phgpu_shim_stats (st)
c.... the residual statistics of solmfg.f:367
        call rstat (res, ilwork)
        end
c
        subroutine ElmGMRs (y,         ac,        x,
     &                     shp,       shgl,      iBC,
     &                     BC,        shpb,      shglb,
     &                     res,       rmes,      BDiag,
     &                     iper,      ilwork,    lhsK,
     &                     col,       row,       rerr)
        use phgpu_shim_state
        include "common.h"
        dimension y(nshg,ndof),         ac(nshg,ndof),
     &            x(numnp,nsd),         iBC(nshg),
     &            BC(nshg,ndofBC),      res(nshg,nflow),
     &            rmes(nshg,nflow),     BDiag(nshg,nflow,nflow),
     &            iper(nshg),           ilwork(nlwork)
        dimension shp(MAXTOP,maxsh,MAXQPT),
     &            shgl(MAXTOP,nsd,maxsh,MAXQPT),
     &            shpb(MAXTOP,maxsh,MAXQPT),
     &            shglb(MAXTOP,nsd,maxsh,MAXQPT)
        integer col(nshg+1), row(nnz*nshg)
        real*8  lhsK(nflow*nflow,nnz_tot), rerr(nshg,10)
        type(c_ptr) ctx
        integer(c_int) :: rc
        call phgpu_shim_setup (x, iBC, BC, iper, ctx)
        rc = phgpu_elmgmrs (ctx, y, ac, res, BDiag, lhsK)
        if (rc .ne. PHGPU_OK) call error ('ElmGMRs ', 'phgpu   ', rc)
        end
c
        subroutine SolGMRs(y,         ac,        yold,      acold,
     &                     x,         iBC,       BC,
     &                     col,       row,       lhsk,
     &                     res,       BDiag,     HBrg,      eBrg,
     &                     yBrg,      Rcos,      Rsin,      iper,
     &                     ilwork,    shp,       shgl,      shpb,
     &                     shglb,     Dy,        rerr)
        use phgpu_shim_state
        include "common.h"
        dimension y(nshg,ndof),         ac(nshg,ndof),
     &            yold(nshg,ndof),      acold(nshg,ndof),
     &            x(numnp,nsd),         iBC(nshg),
     &            BC(nshg,ndofBC),      res(nshg,nflow),
     &            BDiag(nshg,nflow,nflow),
     &            HBrg(Kspace+1,Kspace), eBrg(Kspace+1),
     &            yBrg(Kspace),         Rcos(Kspace),
     &            Rsin(Kspace),         iper(nshg),
     &            ilwork(nlwork),       Dy(nshg,nflow)
        dimension shp(MAXTOP,maxsh,MAXQPT),
     &            shgl(MAXTOP,nsd,maxsh,MAXQPT),
     &            shpb(MAXTOP,maxsh,MAXQPT),
     &            shglb(MAXTOP,nsd,maxsh,MAXQPT)
        integer col(nshg+1), row(nnz*nshg)
        real*8  lhsk(nflow*nflow,nnz_tot), rerr(nshg,10)
        real*8  rmes(nshg,nflow)
        type(c_ptr) ctx
        type(phgpu_stats) :: st
        integer(c_int) :: rc
        call phgpu_shim_setup (x, iBC, BC, iper, ctx)
        st%ntotGM = ntotGM
c.... the COMMON lGMRES that the reference's restart test reads (solgmr.f:528)
        st%lGMRES = lGMRES
        rc = phgpu_solgmrs (ctx, y, ac, lhs, res, BDiag, Dy, lhsk, st)
        if (rc .ne. PHGPU_OK) call error ('SolGMRs ', 'phgpu   ', rc)
        iKs = st%iKs
        ntotGM = st%ntotGM
        lGMRESs = st%lGMRES
c.... the residual statistics of solgmr.f:725
        rmes = zero
        call rstat (res, ilwork, rmes)
        end
c
        subroutine ElmGMRe (y,         ac,        x,
     &                     shp,       shgl,      iBC,
     &                     BC,        shpb,      shglb,
     &                     res,       rmes,      BDiag,
     &                     iper,      ilwork,    EGmass, rerr)
        use phgpu_shim_state
        include "common.h"
        dimension y(nshg,ndof),         ac(nshg,ndof),
     &            x(numnp,nsd),         iBC(nshg),
     &            BC(nshg,ndofBC),      res(nshg,nflow),
     &            rmes(nshg,nflow),     BDiag(nshg,nflow,nflow),
     &            iper(nshg),           ilwork(nlwork),
     &            EGmass(numel,nedof,nedof)
        dimension shp(MAXTOP,maxsh,MAXQPT),
     &            shgl(MAXTOP,nsd,maxsh,MAXQPT),
     &            shpb(MAXTOP,maxsh,MAXQPT),
     &            shglb(MAXTOP,nsd,maxsh,MAXQPT)
        real*8  rerr(nshg,10)
        type(c_ptr) ctx
        integer(c_int) :: rc
        call phgpu_shim_setup (x, iBC, BC, iper, ctx)
        rc = phgpu_elmgmre (ctx, y, ac, res, BDiag, EGmass)
        if (rc .ne. PHGPU_OK) call error ('ElmGMRe ', 'phgpu   ', rc)
        end
c
        subroutine SolGMRe (y,         ac,        yold,      acold,
     &                     x,         iBC,       BC,        EGmass,
     &                     res,       BDiag,     HBrg,      eBrg,
     &                     yBrg,      Rcos,      Rsin,      iper,
     &                     ilwork,    shp,       shgl,      shpb,
     &                     shglb,     Dy, rerr)
        use phgpu_shim_state
        include "common.h"
        dimension y(nshg,ndof),         ac(nshg,ndof),
     &            yold(nshg,ndof),      acold(nshg,ndof),
     &            x(numnp,nsd),         iBC(nshg),
     &            BC(nshg,ndofBC),      EGmass(numel,nedof,nedof),
     &            res(nshg,nflow),      BDiag(nshg,nflow,nflow),
     &            HBrg(Kspace+1,Kspace), eBrg(Kspace+1),
     &            yBrg(Kspace),         Rcos(Kspace),
     &            Rsin(Kspace),         iper(nshg),
     &            ilwork(nlwork),       Dy(nshg,nflow)
        dimension shp(MAXTOP,maxsh,MAXQPT),
     &            shgl(MAXTOP,nsd,maxsh,MAXQPT),
     &            shpb(MAXTOP,maxsh,MAXQPT),
     &            shglb(MAXTOP,nsd,maxsh,MAXQPT)
        real*8  rerr(nshg,10), rmes(nshg,nflow)
        type(c_ptr) ctx
        type(phgpu_stats) :: st
        integer(c_int) :: rc
        call phgpu_shim_setup (x, iBC, BC, iper, ctx)
        st%ntotGM = ntotGM
        rc = phgpu_solgmre (ctx, y, ac, res, BDiag, Dy, EGmass, st)
        if (rc .ne. PHGPU_OK) call error ('SolGMRe ', 'phgpu   ', rc)
        iKs = st%iKs
        ntotGM = st%ntotGM
c.... the residual statistics of solgmr.f:352
        rmes = zero
        call rstat (res, ilwork, rmes)
        end
