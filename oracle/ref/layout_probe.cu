// Prints the byte layout of the reference's ArrayDev3D<double> (the kernel
// parameter type of its compact-derivative and divergence kernels) as a C
// header, so the harness can pass such parameters to the reference's own
// kernels.  Compiled against the reference's header where it lies; run on the
// build host (x86-64 and aarch64 Linux share the LP64 Itanium C++ layout).
#include <cstdio>
#define private public
#define protected public
#include "Engine/cuArray.hpp"
#undef private
#undef protected

int main() {
    ArrayDev3D<double> a;
    const char *base = reinterpret_cast<const char *>(&a);
    printf("/* generated by oracle/ref/layout_probe.cu */\n");
    printf("#define REF_ARRAYDEV3D_SIZE %zu\n", sizeof(a));
    printf("#define REF_ARRAYDEV3D_ALIGN %zu\n", alignof(ArrayDev3D<double>));
    printf("#define REF_OFF_DDATA %td\n", reinterpret_cast<const char *>(&a.d_data) - base);
    printf("#define REF_OFF_DIMSIZE %td\n", reinterpret_cast<const char *>(&a.dimsize) - base);
    printf("#define REF_OFF_NX %td\n", reinterpret_cast<const char *>(&a.nx) - base);
    printf("#define REF_OFF_NY %td\n", reinterpret_cast<const char *>(&a.ny) - base);
    printf("#define REF_OFF_NZ %td\n", reinterpret_cast<const char *>(&a.nz) - base);
    return 0;
}
