// hjm_adjoint.cu -- pathwise adjoint of the CVA (reverse sweep kernels).
#include <cuda_runtime.h>

#include "hjm_kernels.h"
