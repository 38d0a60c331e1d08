/* ORACLE BUILD SHIM (test infrastructure only): see ContinuousStructure.h. */
#include "ContinuousStructure.h"
