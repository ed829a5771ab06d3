/* Empty stand-in: the reference includes <cuda.h> but uses no driver API. */
#include "cuda_runtime.h"
