/* ORACLE BUILD SHIM (test infrastructure only): openEMS includes this Boost header but uses
   nothing from it on the engine path (Boost is not installed in this image). */
#pragma once
