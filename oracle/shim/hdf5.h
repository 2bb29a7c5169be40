/*
 * Stand-in for <hdf5.h>, used ONLY to compile the reference library from its own
 * sources for the oracle (oracle/_ref).  The reference's src/util.h includes
 * <hdf5.h> for its result-file helpers (src/util.c:56-236); none of those helpers
 * is on the evaluation path this project checks, so every call here fails with -1.
 *
 * Test infrastructure: never linked into the product library.
 */
#pragma once

/* the real header brings these in, and the reference's util.c relies on that */
#include <stdio.h>
#include <stdint.h>
#include <inttypes.h>

typedef int64_t hid_t;
typedef int herr_t;
typedef unsigned long long hsize_t;

#define H5P_DEFAULT        ((hid_t)0)
#define H5S_ALL            ((hid_t)0)
#define H5S_SCALAR         ((hid_t)0)
#define H5P_DATASET_CREATE ((hid_t)0)
#define H5F_ACC_RDONLY     0u
#define H5F_ACC_TRUNC      0u
#define H5T_NATIVE_DOUBLE  ((hid_t)1)
#define H5T_NATIVE_INT     ((hid_t)2)
#define H5T_NATIVE_LONG    ((hid_t)3)
#define H5T_IEEE_F64LE     ((hid_t)4)
#define H5T_STD_I32LE      ((hid_t)5)

static inline hid_t H5Dopen(hid_t f, const char* n, hid_t p) { (void)f; (void)n; (void)p; return -1; }
static inline hid_t H5Dget_space(hid_t d) { (void)d; return -1; }
static inline int H5Sget_simple_extent_ndims(hid_t s) { (void)s; return -1; }
static inline int H5Sget_simple_extent_dims(hid_t s, hsize_t* d, hsize_t* m) { (void)s; (void)d; (void)m; return -1; }
static inline herr_t H5Sclose(hid_t s) { (void)s; return -1; }
static inline herr_t H5Dclose(hid_t d) { (void)d; return -1; }
static inline herr_t H5Dread(hid_t d, hid_t t, hid_t ms, hid_t fs, hid_t p, void* b) { (void)d; (void)t; (void)ms; (void)fs; (void)p; (void)b; return -1; }
static inline herr_t H5Dwrite(hid_t d, hid_t t, hid_t ms, hid_t fs, hid_t p, const void* b) { (void)d; (void)t; (void)ms; (void)fs; (void)p; (void)b; return -1; }
static inline hid_t H5Aopen(hid_t o, const char* n, hid_t p) { (void)o; (void)n; (void)p; return -1; }
static inline herr_t H5Aread(hid_t a, hid_t t, void* b) { (void)a; (void)t; (void)b; return -1; }
static inline herr_t H5Awrite(hid_t a, hid_t t, const void* b) { (void)a; (void)t; (void)b; return -1; }
static inline herr_t H5Aclose(hid_t a) { (void)a; return -1; }
static inline hid_t H5Screate_simple(int r, const hsize_t* d, const hsize_t* m) { (void)r; (void)d; (void)m; return -1; }
static inline hid_t H5Screate(hid_t t) { (void)t; return -1; }
static inline hid_t H5Pcreate(hid_t c) { (void)c; return -1; }
static inline herr_t H5Pset_obj_track_times(hid_t p, int b) { (void)p; (void)b; return -1; }
static inline hid_t H5Dcreate(hid_t f, const char* n, hid_t t, hid_t s, hid_t a, hid_t b, hid_t c) { (void)f; (void)n; (void)t; (void)s; (void)a; (void)b; (void)c; return -1; }
static inline hid_t H5Acreate(hid_t f, const char* n, hid_t t, hid_t s, hid_t a, hid_t b) { (void)f; (void)n; (void)t; (void)s; (void)a; (void)b; return -1; }
static inline hid_t H5Fopen(const char* n, unsigned f, hid_t p) { (void)n; (void)f; (void)p; return -1; }
static inline herr_t H5Fclose(hid_t f) { (void)f; return -1; }
