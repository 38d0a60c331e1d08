/*
 * ORACLE BUILD SHIM -- test infrastructure only.  Stand-in for Boost.Predef, which is not
 * installed in this image: only the architecture/endianness macros that openEMS's engine sources
 * test (tools/denormal.h, FDTD/engine_sse_compressed.cpp), derived from the compiler's own macros.
 */
#ifndef OEMS_SHIM_BOOST_PREDEF_H
#define OEMS_SHIM_BOOST_PREDEF_H
/* OEMS_SHIM_ARCH_NOT_X86 builds the reference as it is built for arm64: Denormal::Disable() is
 * then a no-op (tools/denormal.h), so denormals are kept, as on the GPU machines' hosts */
#if (defined(__x86_64__) || defined(__i386__)) && !defined(OEMS_SHIM_ARCH_NOT_X86)
#define BOOST_ARCH_X86 1
#else
#define BOOST_ARCH_X86 0
#endif
#if defined(__powerpc64__)
#define BOOST_ARCH_PPC_64 1
#else
#define BOOST_ARCH_PPC_64 0
#endif
#if defined(__BYTE_ORDER__) && __BYTE_ORDER__ == __ORDER_LITTLE_ENDIAN__
#define BOOST_ENDIAN_LITTLE_BYTE 1
#else
#define BOOST_ENDIAN_LITTLE_BYTE 0
#endif
#endif
