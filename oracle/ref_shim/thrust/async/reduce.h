/* Stand-in for <thrust/async/reduce.h>, which the reference includes
 * (main.cu:15) and CUDA 13's CCCL no longer ships; the reference uses nothing
 * from it.  oracle/ref_cuda.sh puts oracle/ref_shim first on the include path of
 * the reference build, so the reference file itself is compiled unchanged. */
#pragma once
#include <thrust/reduce.h>
