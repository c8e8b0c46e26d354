// Shim for Source/EBR.H: the point-kernel headers include it only for the
// AMReX namespace and NUM_GROW; the AmrLevel class itself is not needed.
#ifndef OCFD_SHIM_EBR_H
#define OCFD_SHIM_EBR_H
#include "amrex_shim.H"
using namespace amrex;
#endif
