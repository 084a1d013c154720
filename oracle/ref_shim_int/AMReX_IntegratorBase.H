/* ORACLE (test infrastructure only): the AMReX header rkn.h includes; the
 * names it needs come from the MultiFab stand-in. */
#include "AMReX_MultiFab.H"
