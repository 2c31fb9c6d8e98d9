// Batched persistent step over many lattices (filled in below).
#include "internal.cuh"
