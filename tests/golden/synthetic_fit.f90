! A made-up inverse-power fit in the layout of the Select_Pot registry:
! the Select_Pot branch, the BLOCK DATA of its COMMON and the evaluating
! function.  It exercises the reader of ep_select_pot without the reference
! source: Real*16 Pg with a Q, a D and an unsuffixed (default REAL) literal,
! continuation lines, comments and a second name that is not a fit.
Double Precision Function Select_Pot(selec,r,r_cutoff,umax)
Implicit None
Character (Len=80) :: selec
Real (Kind=8) :: r, r_cutoff, umax
Real (Kind=8) :: V_test_fit, V_other   ! two candidates
If(Trim(selec).Eq.'Other')Then
   Select_pot = V_other(r)
   Return
ElseIf(Trim(selec).Eq.'Test_fit'.Or.   &
       Trim(selec).Eq.'Test_fit_alias')Then
   If(r.lt.r_cutoff)Then
     Select_pot = umax
   Else
     Select_pot = V_test_fit(r)
   Endif
   Return
ElseIf(Trim(selec).Eq.'Test_even')Then
   Select_pot = V_test_even(r)
   Return
ElseIf(Trim(selec).Eq.'Test_exp')Then
   Select_pot = V_test_exp(r)
   Return
Endif
End Function Select_Pot
Block Data Inicio_LJ_test_fit
Implicit Real*8(A-H,O-Z)
Parameter(Npg=4)
Real*16 Pg
Integer*4 k0
Common/Param_LJ_test_fit/rcutoff,fcutoff,r0,aa,bb,cc,Pg(Npg),k0
Data Pg/                           &
 -2.5000000000000000000000000000001Q4,  1.0Q6,   &
 -0.1, 3.0D6 /
Data rcutoff/ 1.5D0/
Data fcutoff/ 4.0D3/
Data r0/ 2.0D0/
Data aa/ -1.0D3/
Data bb/ 0.0D0/
Data cc/ 8.0D3/
Data k0/   3/
End
Double Precision Function V_test_fit(x)
Parameter(Npg=4)
Implicit Real*8(A-H,O-Z)
Real*16 Pg,Sto,xq,Aux
Integer*4 k0
Common/Param_LJ_test_fit/rcutoff,fcutoff,r0,aa,bb,cc,Pg(Npg),k0
If(x.le.rcutoff)Then
  V_test_fit=fcutoff
  Return
Endif
If(x.le.r0)Then
  V_test_fit=Abs(aa*x**2+bb*x+cc)
  Return
Endif
Sto=0.0q0
xq=1.0q0/x
Aux=xq**(k0+1)
Do k=1,Npg
  Sto=Sto+pg(k)*Aux
  Aux=Aux*xq
EndDo
V_test_fit=Sto
Return
End
Double Precision Function V_other(r)
Implicit None
Real (Kind=8) :: r
V_other = 1.d0/r
End
      Double Precision Function V_test_even(x)
      Implicit Real*8(A-H,O-Z)
      V_test_even=Func_test_even(x)
      Return
      End
      Block Data Inicio_test_even
      Implicit Real*8(A-H,O-Z)
      Parameter(Npg=3)
      Common/Param_test_even/r0,aa,bb,cc,Pg(Npg)
      Data Pg/ -2.0D+03, 5.0D+04, -1.0D+05 /
      Data r0/ 2.0D0/
      Data aa/ 10.0D0/
      Data bb/ -5.0D0/
      Data cc/ 100.0D0/
      End
      Double Precision Function Func_test_even(x)
      Parameter(Npg=3)
      Implicit Real*8(A-H,O-Z)
      Common/Param_test_even/r0,aa,bb,cc,Pg(Npg)
      If(x.le.r0)Then
        Func_test_even=aa*x**2+bb*x+cc
        Return
      Endif
      Sto=0.0d0
      Do k=1,Npg
        Sto=Sto+pg(k)/x**(2*(k-1)+6)
      EndDo
      Func_test_even=Sto
      Return
      End
      Block Data Inicio_test_exp
      Implicit Real*8(A-H,O-Z)
      Parameter(Npg=3)
      Common/Param_test_exp/r0,aa,bb,cc,Pg(Npg),Ps(Npg)
      Data Pg/ 3.0D+03, -1.0D+01, 2.0D-01 /
      Data Ps/ 1.5D+00, 0.5D+00, 0.25D+00 /
      Data r0/ 2.5D0/
      Data aa/ 1.0D0/
      Data bb/ 0.0D0/
      Data cc/ 50.0D0/
      End
      Double Precision Function V_test_exp(xx)
      Parameter(Npg=3)
      Implicit Real*8(A-H,O-Z)
      Common/Param_test_exp/r0,aa,bb,cc,Pg(Npg),Ps(Npg)
      data x0/2.0d0/
      If(xx.lt.x0)then
        x=x0
      Else
         x=xx
      Endif
      If(x.le.r0)Then
        V_test_exp=aa*x**2+bb*x+cc
        Return
      Endif
      Sto=pg(1)*Dexp(-Ps(1)*x)/x
      Do k=2,Npg
        Sto=Sto+pg(k)*x**(k-1)*Dexp(-Ps(k)*x)
      EndDo
      V_test_exp=Sto
      Return
      End
