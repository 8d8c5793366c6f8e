/* Empty stand-in for <cuda_runtime.h> in the CPU build of the reference
 * kernels (see ../refshim/shim.h). */
#pragma once
