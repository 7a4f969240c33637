/*
 * libmexshim.so: host emulation of the MEX API declared in mex.h.
 *
 * An mxArray is a header plus a zero-filled, column-major data block.
 * mexErrMsgTxt unwinds with longjmp to the thread's active mexshim_call(),
 * which frees the arrays created since the call began and reports the
 * message; this is how Matlab itself treats an error raised inside a mex
 * function (outputs discarded, control back to the caller).
 */
#include "mex.h"

#include <setjmp.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define MEXSHIM_MAX_DIMS 8

struct mxArray_tag {
    mxClassID classid;
    mwSize ndim;
    mwSize dims[MEXSHIM_MAX_DIMS];
    size_t numel;
    void *data;
    struct mxArray_tag *next_created; /* per-call allocation list */
};

typedef struct call_frame {
    jmp_buf env;
    char message[1024];
    mxArray *created;
    struct call_frame *outer;
} call_frame;

static _Thread_local call_frame *g_frame = NULL;
static _Thread_local char g_last_print[1024];

static size_t class_size(mxClassID c)
{
    switch (c) {
    case mxDOUBLE_CLASS: return 8;
    case mxSINGLE_CLASS: return 4;
    case mxINT8_CLASS: case mxUINT8_CLASS: return 1;
    case mxINT16_CLASS: case mxUINT16_CLASS: return 2;
    case mxINT32_CLASS: case mxUINT32_CLASS: return 4;
    default: return 0;
    }
}

mxArray *mxCreateNumericArray(mwSize ndim, const mwSize *dims,
                              mxClassID classid, mxComplexity flag)
{
    (void)flag;
    size_t esz = class_size(classid);
    if (esz == 0 || ndim < 0 || ndim > MEXSHIM_MAX_DIMS)
        return NULL;
    mxArray *a = (mxArray *)calloc(1, sizeof(mxArray));
    if (!a)
        return NULL;
    a->classid = classid;
    a->ndim = ndim < 2 ? 2 : ndim;
    a->dims[0] = a->dims[1] = 1;
    size_t numel = 1;
    for (int d = 0; d < ndim; ++d) {
        mwSize n = dims[d] < 0 ? 0 : dims[d];
        a->dims[d] = n;
        numel *= (size_t)n;
    }
    a->numel = numel;
    size_t bytes = numel * esz;
    if (bytes < 8)
        bytes = 8;
    a->data = calloc(1, bytes);
    if (!a->data) {
        free(a);
        return NULL;
    }
    if (g_frame) {
        a->next_created = g_frame->created;
        g_frame->created = a;
    }
    return a;
}

void mxDestroyArray(mxArray *pa)
{
    if (!pa)
        return;
    free(pa->data);
    free(pa);
}

void *mxGetData(const mxArray *pa) { return pa ? pa->data : NULL; }
size_t mxGetNumberOfElements(const mxArray *pa) { return pa ? pa->numel : 0; }
mwSize mxGetNumberOfDimensions(const mxArray *pa) { return pa ? pa->ndim : 0; }
const mwSize *mxGetDimensions(const mxArray *pa) { return pa ? pa->dims : NULL; }
mxClassID mxGetClassID(const mxArray *pa) { return pa ? pa->classid : mxUNKNOWN_CLASS; }

int mexPrintf(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    int n = vsnprintf(g_last_print, sizeof g_last_print, fmt, ap);
    va_end(ap);
    if (getenv("MEXSHIM_VERBOSE"))
        fputs(g_last_print, stdout);
    return n;
}

const char *mexshim_last_print(void) { return g_last_print; }

void mexErrMsgTxt(const char *msg)
{
    if (!g_frame) {
        fprintf(stderr, "mexErrMsgTxt outside mexshim_call: %s\n", msg);
        abort();
    }
    snprintf(g_frame->message, sizeof g_frame->message, "%s", msg ? msg : "");
    longjmp(g_frame->env, 1);
}

int mexshim_call(mexshim_entry fn, int nlhs, mxArray *plhs[], int nrhs,
                 const mxArray *prhs[], char *errbuf, size_t errlen)
{
    call_frame frame;
    memset(&frame, 0, sizeof frame);
    frame.outer = g_frame;
    g_frame = &frame;
    int failed = 0;
    if (setjmp(frame.env) == 0) {
        fn(nlhs, plhs, nrhs, prhs);
    } else {
        failed = 1;
    }
    g_frame = frame.outer;
    if (failed) {
        mxArray *a = frame.created;
        while (a) {
            mxArray *next = a->next_created;
            mxDestroyArray(a);
            a = next;
        }
        for (int i = 0; i < nlhs; ++i)
            plhs[i] = NULL;
        if (errbuf && errlen)
            snprintf(errbuf, errlen, "%s", frame.message);
        return 1;
    }
    /* Successful call: the caller owns every array it received. */
    if (errbuf && errlen)
        errbuf[0] = '\0';
    return 0;
}
