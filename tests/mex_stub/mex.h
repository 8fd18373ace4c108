/* Declarations of the documented MATLAB MEX C API (R2018a interleaved
 * complex) that gpe_mex.cpp uses, for a compile check of the gateway where
 * MATLAB is absent.  This is not MATLAB's header: types are stand-ins with the
 * documented signatures, nothing is linked or run. */
#pragma once
#include <stddef.h>
#include <stdint.h>
typedef size_t mwSize;
typedef size_t mwIndex;
struct mxArray_tag;
typedef struct mxArray_tag mxArray;
typedef struct { double real, imag; } mxComplexDouble;
typedef struct { float real, imag; } mxComplexSingle;
typedef enum { mxUNKNOWN_CLASS, mxDOUBLE_CLASS, mxSINGLE_CLASS, mxUINT64_CLASS } mxClassID;
typedef enum { mxREAL, mxCOMPLEX } mxComplexity;
bool mxIsUint64(const mxArray*);
bool mxIsDouble(const mxArray*);
bool mxIsComplex(const mxArray*);
bool mxIsSingle(const mxArray*);
size_t mxGetNumberOfElements(const mxArray*);
void mexErrMsgIdAndTxt(const char*, const char*, ...);
void mexWarnMsgIdAndTxt(const char*, const char*, ...);
void mxSetM(mxArray*, mwSize);
int mxGetString(const mxArray*, char*, mwSize);
double* mxGetDoubles(const mxArray*);
mxComplexDouble* mxGetComplexDoubles(const mxArray*);
mxComplexSingle* mxGetComplexSingles(const mxArray*);
mxArray* mxCreateDoubleMatrix(mwSize, mwSize, mxComplexity);
mxArray* mxCreateNumericArray(mwSize, const mwSize*, mxClassID, mxComplexity);
mxArray* mxCreateNumericMatrix(mwSize, mwSize, mxClassID, mxComplexity);
void mxDestroyArray(mxArray*);
mxArray* mxCreateDoubleScalar(double);
double mxGetScalar(const mxArray*);
mxArray* mxGetProperty(const mxArray*, mwIndex, const char*);
int mexCallMATLAB(int, mxArray**, int, mxArray**, const char*);
mwSize mxGetNumberOfDimensions(const mxArray*);
const mwSize* mxGetDimensions(const mxArray*);
void* mxGetData(const mxArray*);
