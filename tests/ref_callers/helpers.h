/*
 * Prototypes of the helpers that dtFFT's C and C++ integration programs call
 * (the interface of tests/c/test_utils.h in the reference, CUDA build),
 * implemented in dtfft_test_helpers.c.  Test infrastructure.
 */
#ifndef GB_REF_CALLER_HELPERS_H
#define GB_REF_CALLER_HELPERS_H

#include <stddef.h>
#include <stdint.h>

#include "dtfft.h"

#ifdef __cplusplus
extern "C" {
#endif

void setTestValuesComplexDouble(void*, size_t);
void setTestValuesComplexFloat(void*, size_t);
void setTestValuesDouble(void*, size_t);
void setTestValuesFloat(void*, size_t);
void createGridDims(int32_t, int32_t*, int32_t*, int32_t*, int32_t*);
void attach_gpu_to_process(void);
void scaleFloat(int32_t, void*, size_t, size_t, int32_t, dtfft_stream_t);
void scaleDouble(int32_t, void*, size_t, size_t, int32_t, dtfft_stream_t);
void scaleComplexFloat(int32_t, void*, size_t, size_t, int32_t, dtfft_stream_t);
void scaleComplexDouble(int32_t, void*, size_t, size_t, int32_t, dtfft_stream_t);
void complexDoubleH2D(void*, void*, size_t, int32_t);
void complexFloatH2D(void*, void*, size_t, int32_t);
void doubleH2D(void*, void*, size_t, int32_t);
void floatH2D(void*, void*, size_t, int32_t);
void checkAndReportComplexDouble(size_t, double, double, void*, size_t, void*, int32_t);
void checkAndReportComplexFloat(size_t, double, double, void*, size_t, void*, int32_t);
void checkAndReportDouble(size_t, double, double, void*, size_t, void*, int32_t);
void checkAndReportFloat(size_t, double, double, void*, size_t, void*, int32_t);

#ifdef __cplusplus
}
#endif
#endif
