! mcmod_synth9.f90 -- the synthetic 9-atom surface as a reference PES module
! (the interface of mcmod_waterdimer.f90:1-105): pair Morse network plus the
! quartic double well B((s/s0)^2 - 1)^2 in s = |r_H - r_O1| - |r_H - r_O2|.
! V_init reads the parameter vector from pes_params.dat (one number per line,
! the layout libpimdgpu's PG_PES_SYNTH9 takes: npair, (i, j, D, a, r0) x npair
! with 0-based atom indices, iH, iO1, iO2, B, s0).  The device twin is
! pes_synth9 in csrc/pg_device.cuh.  Not compiled on the build machines.
module mcmod_mass
  implicit none
  double precision::               V0, eps2=1.0d-5
  integer::                        atom1=1, atom2=2, atom3=3
  character, allocatable::         label(:)
  integer::                        n, ndim, ndof, natom, xunit, totdof
  logical::                        potforcepresent
  character(len=20)::              basename
  integer::                        npair, iH, iO1, iO2
  integer, allocatable::           pi(:), pj(:)
  double precision, allocatable::  pD(:), pa(:), pr0(:)
  double precision::               Bdw, s0

contains

  subroutine V_init(iproc)
    integer, intent(in):: iproc
    integer:: q
    double precision:: v
    open(77, file="pes_params.dat", status="old")
    read(77,*) v
    npair= nint(v)
    allocate(pi(npair), pj(npair), pD(npair), pa(npair), pr0(npair))
    do q=1, npair
       read(77,*) v
       pi(q)= nint(v) + 1
       read(77,*) v
       pj(q)= nint(v) + 1
       read(77,*) pD(q)
       read(77,*) pa(q)
       read(77,*) pr0(q)
    end do
    read(77,*) v
    iH= nint(v) + 1
    read(77,*) v
    iO1= nint(v) + 1
    read(77,*) v
    iO2= nint(v) + 1
    read(77,*) Bdw
    read(77,*) s0
    close(77)
    potforcepresent=.true.
    V0=0.0d0
  end subroutine V_init

  subroutine potforce(x, grad, energy)
    implicit none
    double precision:: x(:,:), grad(:,:), energy
    double precision:: d(3), r, e, r1, r2, e1(3), e2(3), s, t, dvds
    integer:: q
    energy= 0.0d0
    grad= 0.0d0
    do q=1, npair
       d(:)= x(:,pi(q)) - x(:,pj(q))
       r= sqrt(sum(d**2))
       e= exp(-pa(q)*(r - pr0(q)))
       energy= energy + pD(q)*(1.0d0 - e)**2
       grad(:,pi(q))= grad(:,pi(q)) + 2.0d0*pD(q)*pa(q)*(1.0d0 - e)*e*d(:)/r
       grad(:,pj(q))= grad(:,pj(q)) - 2.0d0*pD(q)*pa(q)*(1.0d0 - e)*e*d(:)/r
    end do
    e1(:)= x(:,iH) - x(:,iO1)
    e2(:)= x(:,iH) - x(:,iO2)
    r1= sqrt(sum(e1**2))
    r2= sqrt(sum(e2**2))
    s= r1 - r2
    t= (s/s0)**2 - 1.0d0
    energy= energy + Bdw*t**2 - V0
    dvds= 4.0d0*Bdw*t*s/s0**2
    grad(:,iH)= grad(:,iH) + dvds*(e1(:)/r1 - e2(:)/r2)
    grad(:,iO1)= grad(:,iO1) - dvds*e1(:)/r1
    grad(:,iO2)= grad(:,iO2) + dvds*e2(:)/r2
  end subroutine potforce

  function V(x)
    implicit none
    double precision:: V, x(:,:)
    double precision, allocatable:: g(:,:)
    allocate(g(ndim, natom))
    call potforce(x, g, V)
    deallocate(g)
  end function V

  subroutine Vprime(x, grad)
    implicit none
    double precision:: x(:,:), grad(:,:), energy
    call potforce(x, grad, energy)
  end subroutine Vprime

  subroutine Vdoubleprime(x, hess)
    implicit none
    double precision:: hess(:,:,:,:), x(:,:), eps
    double precision, allocatable:: gp(:,:), gm(:,:)
    integer:: i, j
    eps= 1d-4
    allocate(gp(ndim, natom), gm(ndim, natom))
    do i=1, ndim
       do j=1, natom
          x(i,j)= x(i,j) + eps
          call Vprime(x, gp)
          x(i,j)= x(i,j) - 2.0d0*eps
          call Vprime(x, gm)
          x(i,j)= x(i,j) + eps
          hess(i,j,:,:)= (gp(:,:) - gm(:,:))/(2.0d0*eps)
       end do
    end do
    deallocate(gp, gm)
  end subroutine Vdoubleprime
end module mcmod_mass
