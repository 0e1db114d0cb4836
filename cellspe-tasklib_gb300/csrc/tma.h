// Host access to the driver's tensor-map encoder (cuTensorMapEncodeTiled),
// resolved once through the runtime's driver entry-point query.
#pragma once
#include <cuda.h>

typedef CUresult (*CsEncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                    const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                    CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
// null when the driver does not provide it
CsEncodeTiledFn cs_encode_tiled();
