/* Empty stand-in: the reference headers include <cuda.h>; the CPU build of
 * the reference kernels needs none of it (see ../refshim/shim.h). */
#pragma once
