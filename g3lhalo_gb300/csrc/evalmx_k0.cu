// Mixed-precision rule kernels of NNMap (kind 0): the three terms in the three
// register-budget variants; split from the NMapMap/NNMap unit so the two compile in parallel.
#include "evalmx_impl.cuh"

namespace g3l {

#define G3L_INSTMX(Tm, MB)                                                                     \
    template __global__ void k_evalmx<0, Tm, MB>(DevTables, const IntDesc *, IntState *, Pool, \
                                                 BatchHdr *, const long long *);
G3L_INSTMX(1, 7)
G3L_INSTMX(1, 6)
G3L_INSTMX(1, 8)
G3L_INSTMX(2, 7)
G3L_INSTMX(2, 6)
G3L_INSTMX(2, 8)
G3L_INSTMX(3, 7)
G3L_INSTMX(3, 6)
G3L_INSTMX(3, 8)

// variant 0, 1, 2 = 7, 6, 8 blocks per SM (72, 80, 64 registers per thread)
void *evalmx_kernel_k0(int term, int variant)
{
    static void *tab[3][3] = {
        {(void *)k_evalmx<0, 1, 7>, (void *)k_evalmx<0, 1, 6>, (void *)k_evalmx<0, 1, 8>},
        {(void *)k_evalmx<0, 2, 7>, (void *)k_evalmx<0, 2, 6>, (void *)k_evalmx<0, 2, 8>},
        {(void *)k_evalmx<0, 3, 7>, (void *)k_evalmx<0, 3, 6>, (void *)k_evalmx<0, 3, 8>}};
    return tab[term - 1][variant];
}

}  // namespace g3l
