/* abi_check.c -- the public headers compile as C99 and the library links
 * from C; the host-side argument checks answer without a GPU. */
#include <stdio.h>

#include "radeonrays.h"
#include "radeonrays_cuda.h"

int main(void)
{
    size_t    sz  = 0;
    RRContext ctx = 0;
    int       bad = 0;
    bad += rrGetTraceMemoryRequirements(0, 1, &sz) != RR_ERROR_INVALID_PARAMETER;
    bad += rrCreateContext(RR_API_VERSION, RR_API_VK, &ctx) != RR_ERROR_UNSUPPORTED_API;
    bad += rrCreateContext(RR_API_VERSION, RR_API_CUDA, 0) != RR_ERROR_INVALID_PARAMETER;
    bad += rrCmdIntersect(0, 0, RR_INTERSECT_QUERY_CLOSEST, 0, 1, 0, RR_INTERSECT_QUERY_OUTPUT_FULL_HIT, 0, 0, 0) !=
           RR_ERROR_INVALID_PARAMETER;
    bad += sizeof(RRRay) != 32 || sizeof(RRHit) != 16 || sizeof(RRInstance) != 56;
    bad += RR_CUDA_NODE_FORMAT_BVH4 != 2 || RR_CUDA_TRAVERSAL_BVH4 != 4;
    if (bad)
    {
        printf("FAIL: %d checks\n", bad);
        return 1;
    }
    printf("ok\n");
    return 0;
}
