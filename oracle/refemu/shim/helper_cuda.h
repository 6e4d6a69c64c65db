/* Stand-in for the CUDA samples' helper_cuda.h: checkCudaErrors and
 * getLastCudaError as the reference uses them (abort on a non-zero status). */
#ifndef OSE_REFEMU_HELPER_CUDA_H
#define OSE_REFEMU_HELPER_CUDA_H
#include <stdio.h>
#include <stdlib.h>
#include <cuda_runtime_api.h>
template <typename T>
static inline void refemu_check(T result, const char* what, const char* file, int line)
{
    if ((int)result != 0) {
        fprintf(stderr, "refemu: %s failed with %d at %s:%d\n", what, (int)result, file, line);
        exit(3);
    }
}
#define checkCudaErrors(val) refemu_check((val), #val, __FILE__, __LINE__)
#define getLastCudaError(msg) refemu_check(cudaGetLastError(), msg, __FILE__, __LINE__)
#endif
