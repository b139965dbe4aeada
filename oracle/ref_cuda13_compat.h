/* Force-included when compiling the reference's host helpers with CUDA 13:
 * three cufftResult values used by the reference's error-string table
 * (include/cufinufft_errors.h:29,33,39) were removed from cufft.h. */
#include <cufft.h>
#define CUFFT_INCOMPLETE_PARAMETER_LIST ((cufftResult_t)10)
#define CUFFT_PARSE_ERROR ((cufftResult_t)12)
#define CUFFT_LICENSE_ERROR ((cufftResult_t)15)
