/*
 * kernels_coop.cu -- K4c: the block-cooperative grouped batched IAS15 (the
 * default batched kernel), its builds and launchers.  The kernel itself is
 * in ias15_coop.cuh; the IAS15 pieces it shares with the independent and
 * warp-grouped kernels are in ias15_common.cuh.  A translation unit of its
 * own so that its builds compile beside kernels_ias15.cu.
 */
#include <cuda_runtime.h>
#include <cmath>
#include <cstdio>

#include <type_traits>

#include "device_forces.cuh"
#include "ias15_common.cuh"
#include "internal.h"
#include "warp_table.cuh"
#include "mlp.cuh"

#include "ias15_coop.cuh"
