/* Declarations of the documented mxGPUArray API (MATLAB Parallel Computing
 * Toolbox, gpu/mxGPUArray.h) that gpe_mex.cpp uses, for the compile check of
 * the gateway where MATLAB is absent.  Not MATLAB's header. */
#pragma once
#include "../mex.h"
struct mxGPUArray_tag;
typedef struct mxGPUArray_tag mxGPUArray;
typedef enum { MX_GPU_INITIALIZE_VALUES, MX_GPU_DO_NOT_INITIALIZE } mxGPUInitialize;
int mxInitGPU(void);
const mxGPUArray* mxGPUCreateFromMxArray(const mxArray*);
const void* mxGPUGetDataReadOnly(const mxGPUArray*);
void* mxGPUGetData(mxGPUArray*);
mxClassID mxGPUGetClassID(const mxGPUArray*);
mxComplexity mxGPUGetComplexity(const mxGPUArray*);
mxGPUArray* mxGPUCreateGPUArray(mwSize, const mwSize*, mxClassID, mxComplexity, mxGPUInitialize);
mxArray* mxGPUCreateMxArrayOnGPU(const mxGPUArray*);
void mxGPUDestroyGPUArray(const mxGPUArray*);
