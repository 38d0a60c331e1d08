/* ORACLE BUILD SHIM (test infrastructure only): see vtk_shim.h. */
#include "vtk_shim.h"
