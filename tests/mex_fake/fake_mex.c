/* Fake MATLAB runtime for exercising the MEX shims without MATLAB.  Arrays live in host
 * memory (the library stages host pointers itself); mexErrMsgIdAndTxt unwinds to the
 * harness with longjmp, as MATLAB does.  harness_call() runs mexFunction on arrays described
 * by (ndims, dims, class, data) and returns 0 with the first output copied out, or 1 with
 * the error id and message. */
#include <setjmp.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "gpu/mxGPUArray.h"
#include "mex.h"

struct mxArray_tag {
  mwSize nd;
  mwSize dims[8];
  mxClassID cls;
  void* data;
};
struct mxGPUArray_tag {
  mwSize nd;
  mwSize dims[8];
  mxClassID cls;
  void* data;
  int owns;
};

static jmp_buf g_jmp;
static char g_id[256], g_msg[1024];

void mexErrMsgIdAndTxt(const char* id, const char* fmt, ...) {
  va_list ap;
  snprintf(g_id, sizeof g_id, "%s", id);
  va_start(ap, fmt);
  vsnprintf(g_msg, sizeof g_msg, fmt, ap);
  va_end(ap);
  longjmp(g_jmp, 1);
}
void mxFree(void* p) { free(p); }
int mxInitGPU(void) { return 0; }

static size_t count(mwSize nd, const mwSize* d) {
  size_t n = 1;
  for (mwSize i = 0; i < nd; ++i) n *= d[i];
  return n;
}
const mxGPUArray* mxGPUCreateFromMxArray(const mxArray* a) {
  mxGPUArray* g = (mxGPUArray*)calloc(1, sizeof *g);
  g->nd = a->nd;
  memcpy(g->dims, a->dims, sizeof g->dims);
  g->cls = a->cls;
  g->data = a->data;
  return g;
}
mwSize mxGPUGetNumberOfDimensions(const mxGPUArray* a) { return a->nd; }
const mwSize* mxGPUGetDimensions(const mxGPUArray* a) {
  mwSize* d = (mwSize*)malloc(sizeof(mwSize) * 8);
  memcpy(d, a->dims, sizeof(mwSize) * 8);
  return d;
}
mxClassID mxGPUGetClassID(const mxGPUArray* a) { return a->cls; }
const void* mxGPUGetDataReadOnly(const mxGPUArray* a) { return a->data; }
void* mxGPUGetData(mxGPUArray* a) { return a->data; }
mxGPUArray* mxGPUCreateGPUArray(mwSize nd, const mwSize* dims, mxClassID cls, mxComplexity cx, mxGPUInitialize init) {
  mxGPUArray* g = (mxGPUArray*)calloc(1, sizeof *g);
  (void)cx;
  (void)init;
  g->nd = nd;
  memcpy(g->dims, dims, sizeof(mwSize) * nd);
  g->cls = cls;
  g->data = calloc(count(nd, dims), 4);
  g->owns = 1;
  return g;
}
mxArray* mxGPUCreateMxArrayOnGPU(const mxGPUArray* a) {
  mxArray* m = (mxArray*)calloc(1, sizeof *m);
  m->nd = a->nd;
  memcpy(m->dims, a->dims, sizeof m->dims);
  m->cls = a->cls;
  m->data = malloc(count(a->nd, a->dims) * 4);
  memcpy(m->data, a->data, count(a->nd, a->dims) * 4);
  return m;
}
void mxGPUDestroyGPUArray(const mxGPUArray* a) {
  if (a->owns) free(a->data);
  free((void*)a);
}

int harness_call(int nrhs, const int* nds, const int64_t* dims, const int* classes, void** datas, float* out,
                 size_t out_n, char* id, char* msg) {
  mxArray a[4];
  const mxArray* prhs[4];
  mxArray* plhs[1] = {0};
  for (int k = 0; k < nrhs && k < 4; ++k) {
    memset(&a[k], 0, sizeof a[k]);
    a[k].nd = (mwSize)nds[k];
    for (int d = 0; d < nds[k] && d < 8; ++d) a[k].dims[d] = (mwSize)dims[8 * k + d];
    a[k].cls = (mxClassID)classes[k];
    a[k].data = datas[k];
    prhs[k] = &a[k];
  }
  g_id[0] = g_msg[0] = 0;
  if (setjmp(g_jmp)) {
    snprintf(id, 256, "%s", g_id);
    snprintf(msg, 1024, "%s", g_msg);
    return 1;
  }
  mexFunction(1, plhs, nrhs, prhs);
  if (plhs[0]) {
    const size_t n = count(plhs[0]->nd, plhs[0]->dims);
    memcpy(out, plhs[0]->data, 4 * (n < out_n ? n : out_n));
    free(plhs[0]->data);
    free(plhs[0]);
  }
  return 0;
}
