! mcmod_synth18.f90 -- the synthetic 18-atom water-cluster surface as a
! reference PES module (interface of mcmod_waterdimer.f90:1-105).  Atoms are
! (O, H, H) per molecule; V = sum_m [kr/2 ((r1-re)^2 + (r2-re)^2) + kth/2 (th-the)^2]
! + sum_{m<n} [4 eps ((sig/r_OO)^12 - (sig/r_OO)^6) + sum q_i q_j / r_ij] - V0.
! V_init reads nmol, kr, re, kth, the, eps, sig, qO, qH from pes_params.dat.
! The device twin is pes_synth18 in csrc/pg_device.cuh.  Not compiled here.
module mcmod_mass
  implicit none
  double precision::               V0, eps2=1.0d-5
  integer::                        atom1=1, atom2=2, atom3=3
  character, allocatable::         label(:)
  integer::                        n, ndim, ndof, natom, xunit, totdof
  logical::                        potforcepresent
  character(len=20)::              basename
  integer::                        nmol
  double precision::               kr, re, kth, the, eps, sig, qO, qH

contains

  subroutine V_init(iproc)
    integer, intent(in):: iproc
    double precision:: v
    open(77, file="pes_params.dat", status="old")
    read(77,*) v
    nmol= nint(v)
    read(77,*) kr
    read(77,*) re
    read(77,*) kth
    read(77,*) the
    read(77,*) eps
    read(77,*) sig
    read(77,*) qO
    read(77,*) qH
    close(77)
    potforcepresent=.true.
    V0=0.0d0
  end subroutine V_init

  subroutine potforce(x, grad, energy)
    implicit none
    double precision:: x(:,:), grad(:,:), energy
    double precision:: u1(3), u2(3), r1, r2, ct, st, th, dth, n1(3), n2(3), g1(3), g2(3)
    double precision:: d(3), rr, e, dvr, qa, qb, sr6
    integer:: m, mm, ia, ib, a, b
    energy= 0.0d0
    grad= 0.0d0
    do m=0, nmol-1
       u1(:)= x(:,3*m+2) - x(:,3*m+1)
       u2(:)= x(:,3*m+3) - x(:,3*m+1)
       r1= sqrt(sum(u1**2))
       r2= sqrt(sum(u2**2))
       n1= u1/r1
       n2= u2/r2
       ct= max(-1.0d0, min(1.0d0, sum(n1*n2)))
       th= acos(ct)
       st= max(sqrt(1.0d0 - ct*ct), 1d-12)
       energy= energy + 0.5d0*kr*((r1-re)**2 + (r2-re)**2) + 0.5d0*kth*(th-the)**2
       dth= kth*(th-the)
       g1= kr*(r1-re)*n1 - dth*(n2 - ct*n1)/(r1*st)
       g2= kr*(r2-re)*n2 - dth*(n1 - ct*n2)/(r2*st)
       grad(:,3*m+2)= grad(:,3*m+2) + g1
       grad(:,3*m+3)= grad(:,3*m+3) + g2
       grad(:,3*m+1)= grad(:,3*m+1) - g1 - g2
    end do
    do m=0, nmol-1
       do mm=m+1, nmol-1
          do ia=0, 2
             do ib=0, 2
                a= 3*m + ia + 1
                b= 3*mm + ib + 1
                d(:)= x(:,a) - x(:,b)
                rr= sqrt(sum(d**2))
                qa= qH
                if (ia .eq. 0) qa= qO
                qb= qH
                if (ib .eq. 0) qb= qO
                e= qa*qb/rr
                dvr= -e/rr**2
                if (ia .eq. 0 .and. ib .eq. 0) then
                   sr6= (sig/rr)**6
                   e= e + 4.0d0*eps*(sr6**2 - sr6)
                   dvr= dvr + 4.0d0*eps*(-12.0d0*sr6**2 + 6.0d0*sr6)/rr**2
                end if
                energy= energy + e
                grad(:,a)= grad(:,a) + dvr*d(:)
                grad(:,b)= grad(:,b) - dvr*d(:)
             end do
          end do
       end do
    end do
    energy= energy - V0
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
    double precision:: hess(:,:,:,:), x(:,:), epsfd
    double precision, allocatable:: gp(:,:), gm(:,:)
    integer:: i, j
    epsfd= 1d-4
    allocate(gp(ndim, natom), gm(ndim, natom))
    do i=1, ndim
       do j=1, natom
          x(i,j)= x(i,j) + epsfd
          call Vprime(x, gp)
          x(i,j)= x(i,j) - 2.0d0*epsfd
          call Vprime(x, gm)
          x(i,j)= x(i,j) + epsfd
          hess(i,j,:,:)= (gp(:,:) - gm(:,:))/(2.0d0*epsfd)
       end do
    end do
    deallocate(gp, gm)
  end subroutine Vdoubleprime
end module mcmod_mass
