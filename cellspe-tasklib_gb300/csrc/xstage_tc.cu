// K-d2: X stage on tcgen05 tensor cores (FP16 in, FP32 accumulate).
#include "common.cuh"
#include "kernels.h"

int cs_xmac_tc_f16(const void*, int, int, int, float2*, const float*, int, cudaStream_t)
{
    return CS_ERR_UNSUPPORTED;
}
