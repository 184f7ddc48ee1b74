#!/bin/bash
# Looks for a Fortran compiler able to build Atomistica's Fortran sources
# (the reference of this project).  Prints what it finds; run on a machine
# to record whether oracle/_ref could be built there.
for c in gfortran gfortran-12 gfortran-13 gfortran-14 f95 f77 flang flang-new flang-new-17 \
         flang-new-18 flang-new-19 flang-20 ifx ifort nvfortran lfortran g95; do
  p=$(command -v "$c") && echo "found: $c -> $p"
done
ls /usr/bin | grep -i -E 'fortran|flang|f95|f77' || echo "no Fortran driver in /usr/bin"
find / -xdev \( -name f951 -o -name '*gfortran*' -o -name '*flang*' \) 2>/dev/null | grep -v -E '^/proc|^/sys' | head -20
gcc --version | head -1
echo 'program p; print *, 1; end program' > /tmp/probe_fortran.f90
gcc -c /tmp/probe_fortran.f90 -o /tmp/probe_fortran.o 2>&1 | head -3
uname -m; nproc
