/* Test infrastructure: the few Windows declarations the reference's Muslib
 * sources use, so they compile unchanged with g++ on Linux into the oracle
 * library oracle/_ref/libmuslib_ref.so (never part of the product).
 *
 * Windows is LLP64: long, LONG and ULONG are 32 bits there, and the reference's
 * integer box bounds depend on it (min(long, ULONG) compares as unsigned
 * 32-bit values).  The system headers the sources need are included first,
 * then `long` is mapped to `int` so every long the Muslib sources declare has
 * its Windows width; nothing after this header includes a system header. */
#pragma once
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef uint32_t ULONG;
typedef int32_t LONG;
typedef int BOOL;
typedef uint32_t DWORD;
typedef void *HANDLE;
typedef void *LPVOID;
#define TRUE 1
#define FALSE 0
#define APIENTRY
#define _declspec(x)
#define __declspec(x)
#define min(a, b) (((a) < (b)) ? (a) : (b))
#define max(a, b) (((a) > (b)) ? (a) : (b))
#define long int
