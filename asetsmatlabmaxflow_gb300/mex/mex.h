/*
 * Minimal MEX host API: the subset of Matlab's mex/mx interface that the
 * ASETS mex entry points use (mxGetData, mxCreateNumericArray, mexPrintf,
 * mexErrMsgTxt), plus a few read-only queries.
 *
 * Where Matlab is installed, the drop-in mex sources in this directory are
 * compiled against Matlab's own mex.h with `mex -compatibleArrayDims`
 * instead; this header mirrors that ABI (mwSize == int, the pre
 * largeArrayDims convention the ASETS sources use when they cast
 * `(const int*)dim`, maxflow/asetsBinaryMF2D_mex.c:89).
 *
 * libmexshim.so (mexshim.c) implements it so that mex entry points, both the
 * GPU drop-ins and the reference C solvers, can be called from C or Python
 * without Matlab.
 */
#ifndef ASETS_MEX_SHIM_H
#define ASETS_MEX_SHIM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int mwSize;
typedef struct mxArray_tag mxArray;

/* Class ids carry Matlab's numeric values so dumps and tests can share them. */
typedef enum {
    mxUNKNOWN_CLASS = 0,
    mxDOUBLE_CLASS = 6,
    mxSINGLE_CLASS = 7,
    mxINT8_CLASS = 8,
    mxUINT8_CLASS = 9,
    mxINT16_CLASS = 10,
    mxUINT16_CLASS = 11,
    mxINT32_CLASS = 12,
    mxUINT32_CLASS = 13
} mxClassID;

typedef enum { mxREAL = 0, mxCOMPLEX = 1 } mxComplexity;

/* Zero-filled numeric array.  The allocation is at least 8 bytes even for a
 * 1x1 uint16/single array, because the reference mex files write an int
 * (4 bytes) into the uint16 `i` output and a double into the single `timet`
 * output (maxflow/asetsBinaryMF2D_mex.c:103-111, :125). */
mxArray *mxCreateNumericArray(mwSize ndim, const mwSize *dims,
                              mxClassID classid, mxComplexity flag);
void mxDestroyArray(mxArray *pa);
void *mxGetData(const mxArray *pa);
size_t mxGetNumberOfElements(const mxArray *pa);
mwSize mxGetNumberOfDimensions(const mxArray *pa);
const mwSize *mxGetDimensions(const mxArray *pa);
mxClassID mxGetClassID(const mxArray *pa);

int mexPrintf(const char *fmt, ...);
/* Does not return: unwinds to the enclosing mexshim_call(). */
void mexErrMsgTxt(const char *msg)
#if defined(__GNUC__)
    __attribute__((noreturn))
#endif
    ;

/* ---- host side of the emulation (not part of Matlab's API) ---- */

typedef void (*mexshim_entry)(int nlhs, mxArray *plhs[], int nrhs,
                              const mxArray *prhs[]);

/* Calls `fn` like the Matlab interpreter would.  Returns 0 on success.  If
 * the entry point raised mexErrMsgTxt, returns 1, copies the message into
 * errbuf, and frees every array the call created (as Matlab frees plhs on
 * error).  Thread-safe: the unwind target is thread-local. */
int mexshim_call(mexshim_entry fn, int nlhs, mxArray *plhs[], int nrhs,
                 const mxArray *prhs[], char *errbuf, size_t errlen);

/* Text of the last mexPrintf on this thread (printing to stdout only happens
 * when MEXSHIM_VERBOSE is set in the environment). */
const char *mexshim_last_print(void);

#ifdef __cplusplus
}
#endif

#endif /* ASETS_MEX_SHIM_H */
