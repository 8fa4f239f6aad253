// handle_info.h — what the column-physics entry points (column_kernels.cu)
// need from a chemistry handle, which chem_kernels.cu owns.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

namespace rpb {
struct HandleInfo {
    int device;
    int nlon, nlat, niv, nivbas, nivhau, nrappmax;
    cudaStream_t stream;
};
// REPROBUS_ERR_ARG (with the error text set) when handle is NULL
int handle_info(void* handle, HandleInfo* out);
// device scratch of the handle, grown to at least `bytes` on first need and
// kept until reprobus_chem_free; *out gets its address
int handle_scratch(void* handle, size_t bytes, void** out);
}  // namespace rpb
