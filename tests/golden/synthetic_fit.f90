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
