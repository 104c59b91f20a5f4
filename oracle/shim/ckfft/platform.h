/* Build shim for compiling the reference's sources on Linux (test infrastructure).
 * The reference's own platform header stops with "Unsupported platform" on Linux;
 * placed first on the include path, this header stands in for it.  It selects no
 * OS-specific code (the generic vprintf branch of the reference's debug printer
 * and the scalar FFT path are what get built) and supplies the integer typedefs
 * that the reference's sources expect in namespace ckfft. */
#pragma once
#define CKFFT_PLATFORM_LINUX_SHIM 1
namespace ckfft
{
typedef unsigned char uchar;
typedef unsigned short ushort;
typedef unsigned int uint;
typedef unsigned long ulong;
typedef signed char int8;
typedef unsigned char uint8;
typedef signed short int16;
typedef unsigned short uint16;
typedef signed int int32;
typedef unsigned int uint32;
typedef signed long long int64;
typedef unsigned long long uint64;
}
