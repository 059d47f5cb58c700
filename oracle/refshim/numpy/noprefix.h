/* Legacy numpy alias stub for building the reference's vendored ANUGA C
 * extension against numpy 2.x headers (numpy 2 dropped noprefix.h).  Only the
 * handful of old names that the reference's numpy_shim.h / util_ext.h use are
 * mapped; nothing here is called by the oracle's pure-C entry points. */
#ifndef SWGPU_REFSHIM_NOPREFIX_H
#define SWGPU_REFSHIM_NOPREFIX_H
#define NPY_NO_DEPRECATED_API NPY_1_7_API_VERSION
#include <numpy/arrayobject.h>
#define MAX_DIMS NPY_MAXDIMS
#define CARRAY NPY_ARRAY_CARRAY
#define PyArray_OBJECT NPY_OBJECT
#define PyArray_DOUBLE NPY_DOUBLE
#define PyArray_LONG NPY_LONG
#define PyArray_INT NPY_INT
#endif
