/*
 * Scalar types of the matchgate library (drop-in for the reference's src/config.h:1-55).
 *
 * This library is built for complex circuits only (the reference's COMPLEX_CIRCUIT
 * build, CMakeLists.txt:16); the real-valued variant is not provided.
 */
#pragma once

#include <stdlib.h>
#include <complex.h>

#ifndef COMPLEX_CIRCUIT
#define COMPLEX_CIRCUIT
#endif

/* scalar of gates and state vectors: complex128 (src/config.h:11) */
typedef double complex numeric;

#define _abs cabs

/* alignment of host buffers allocated by this library (src/config.h:29) */
#define MEM_DATA_ALIGN 64

static inline void aligned_free(void* memblock)
{
	free(memblock);
}

/* integer type addressing entries of a state vector (src/config.h:55) */
typedef long int intqs;
