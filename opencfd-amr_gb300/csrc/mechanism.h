// Li-Dryer H2/O2 mechanism data (9 species, 19 reactions) as the kernels use it.
#pragma once

#include "ocfd/ocfd.h"

namespace ocfd {

constexpr int NSP = OCFD_NSPEC;

// Table block mirrored in device constant memory (chem.cu).
struct MechTables {
    double mw[NSP];
    double lo[NSP][7];   // NASA-7 coefficients, T < 1000 K
    double hi[NSP][7];   // NASA-7 coefficients, T >= 1000 K
    double HP[NSP];      // lo[n][5]
    double A0[NSP];      // lo[n][0] - 1
    double visc[NSP * 5];
    double cond[NSP * 5];
    double diff[45 * 5];
};

// The built-in tables (Source/Constants.cpp:15-150).
void mech_builtin(MechTables* t);
// Points the CHEM table members of `p` at the library's host copies of the
// reference's Source/Constants.cpp:15-150 data.
void mech_host_tables(ocfd_parm* p);
// Gathers the tables `p` points at (host or device memory; NULL members fall
// back to the built-in data) and uploads them to constant memory.
ocfd_status mech_upload(const ocfd_parm& p);

}  // namespace ocfd
