// Launch accounting hooks (see timing.cu).
#pragma once
#include <cuda_runtime.h>

namespace dd {
int kt_begin(const char* label, cudaStream_t st);
void kt_end(int slot, cudaStream_t st);
}  // namespace dd

// Wrap one kernel launch: DD_KT(label, stream, kernel<<<...>>>(...));
#define DD_KT(label, st, ...)                    \
    do {                                         \
        int kt_slot_ = ::dd::kt_begin(label, st); \
        __VA_ARGS__;                             \
        ::dd::kt_end(kt_slot_, st);              \
    } while (0)
