// Shim: forwards to the project-written AMReX stand-ins.
#include "amrex_shim.H"
