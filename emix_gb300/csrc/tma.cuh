// tma.cuh -- pieces shared by the kernels that stage tiles with the tensor
// memory accelerator: the driver's tensor-map encoder, the shared-memory
// address of a pointer, the bounded mbarrier wait.
#pragma once

#include "common.cuh"

#include <cudaTypedefs.h>   // PFN_cuTensorMapEncodeTiled

namespace emix {

// cuTensorMapEncodeTiled from the driver, fetched once through the runtime
// (null where the driver does not offer it)
PFN_cuTensorMapEncodeTiled_v12000 tma_encode_fn();

constexpr long kTmaWaitLimit = 1L << 22;            // polls (with 64 ns pauses) before giving up

EMIX_DEV unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

// bounded wait for phase `parity` of the mbarrier at shared address bar:
// non-blocking tests with 64 ns pauses, about 0.3 s in all before giving up
EMIX_DEV bool mbar_wait(unsigned bar, unsigned parity) {
    for (long it = 0; it < kTmaWaitLimit; ++it) {
        unsigned done;
        asm volatile("{\n\t.reg .pred p;\n\t"
                     "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}"
                     : "=r"(done) : "r"(bar), "r"(parity) : "memory");
        if (done) return true;
        __nanosleep(64);
    }
    return false;
}

} // namespace emix
