/* Host-only build of the reference: nothing to declare. */
#pragma once
#include <cuda_runtime.h>
