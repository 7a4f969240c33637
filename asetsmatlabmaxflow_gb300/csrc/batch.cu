// Batched persistent solver (see batch kernels).
#include "internal.h"
