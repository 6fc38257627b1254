"""CPU oracle for the J-VIE solve path -- TEST INFRASTRUCTURE ONLY.

A plain numpy/scipy restatement of the reference MATLAB code on this path
(getOPERATORS -> mv_AN -> pgmres, JVIE_Solver, the excitations, E_field_Nop
and the Mie series), each function citing the reference file:line it follows.
Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may import
it, and only as the checker.  The product (marie_gb300) never calls it.

Parity pins: the reference MATLAB cannot run here (no MATLAB/Octave), so the
matvec and GMRES restatements are pinned by known-answer identities (delta
operator, adjoint identity, dense solves) and by the analytic Mie series; the
operator-assembly restatement is pinned against the reference's own C++ cores
(cubature_nop.cpp and the DIRECTFN singular integrals) built from the
reference sources into oracle/_ref/ (see oracle/Makefile), through golden
fixtures committed under tests/golden/.
"""
