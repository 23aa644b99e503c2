// The tile-pass kernels for float elements (see kernels.cuh).
#include "kernels_impl.cuh"

template struct lsg::PassKernels<float>;
