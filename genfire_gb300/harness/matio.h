/*
 * matio.h -- MAT-file (Level 5) input and output for the standalone harness.
 *
 * Reading covers what readFiles (GENFIRE_Reconstructor.m:82-112) hands to
 * importdata: the first numeric or logical array of a Level-5 MAT file,
 * stored plainly or zlib-compressed (miCOMPRESSED, the default of MATLAB 7+),
 * converted to double.  Writing produces uncompressed Level-5 files of
 * double, single or logical arrays, as save() would for SaveResults.
 * Level-7.3 (HDF5) files are not read.
 */
#ifndef GENFIRE_MATIO_H
#define GENFIRE_MATIO_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    char name[64];      /* variable name */
    int ndims;          /* number of dimensions (>= 2) */
    int64_t dims[8];    /* sizes, column-major */
    int64_t numel;
    int mx_class;       /* MATLAB array class (6 double, 7 single, 8.. integers) */
    int is_logical;
    int is_complex;
    double *re;         /* numel values (column-major), malloc'd */
    double *im;         /* imaginary part or NULL */
} mat_array;

/* Reads the first numeric or logical array of `path` (or the one named `name`
 * if not NULL).  Returns 0 on success; on failure a message is written to
 * err (err_len bytes).  Free with mat_free. */
int mat_read(const char *path, const char *name, mat_array *out, char *err, size_t err_len);
void mat_free(mat_array *a);

/* Element class of a variable to write */
enum { MAT_DOUBLE = 6, MAT_SINGLE = 7, MAT_LOGICAL = 9 };

typedef struct {
    const char *name;
    int ndims;
    const int64_t *dims;
    int mx_class;        /* MAT_DOUBLE (data: double), MAT_SINGLE (float), MAT_LOGICAL (uint8) */
    const void *data;
} mat_var;

/* Writes an uncompressed Level-5 MAT file holding `count` variables. */
int mat_write(const char *path, int count, const mat_var *vars, char *err, size_t err_len);

/* zlib-format decompression (RFC 1950 around RFC 1951 DEFLATE); returns the
 * number of bytes written to out, or -1 on malformed input or overflow. */
int64_t mat_inflate(const uint8_t *in, size_t in_len, uint8_t *out, size_t out_cap);

#ifdef __cplusplus
}
#endif

#endif
