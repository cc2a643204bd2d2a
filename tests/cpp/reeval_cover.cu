// Host check of the FP64 re-take of an unsettled split (split-only entries): for every
// kind, term and mask of contending dimensions, every value a needed rule point reads is
// one the passes compute.  The passes compute, for a split-only entry with mask cm
// (eval_fp64.cu: k_re_fill, k_re_ucache, k_re_points, k_reeval64):
//   - coordinate slots (dim, v) with split_variant(cm, dim, v);
//   - (mass, z) pairs with at most one of vm, vz non-zero and both split_variant;
//   - (l, m, z) u_NFW combinations with at most one non-zero variant, each split_variant;
//   - k3 u_NFW and auxiliary projections whose first point passes split_point;
//   - the points that pass split_point.
// The needed points are the centre and the contenders' axis points.  Prints "ok <n>" and
// exits 0, or prints the first failure and exits 1.
#include <cstdio>

#include "g3l_device.cuh"

using namespace g3l;

static int first_of(const uint32_t *code, int p, uint32_t keep)
{
    int q = 0;
    while ((code[q] & keep) != (code[p] & keep)) ++q;
    return q;
}

static bool pair_computed(unsigned cm, int md, int zd, int vm, int vz)
{
    return !(vm && vz) && split_variant(cm, md, vm) && split_variant(cm, zd, vz) &&
           mz_vm_of(mz_index(vm, vz)) == vm && mz_vz_of(mz_index(vm, vz)) == vz;
}

#define FAIL(...)                                                                        \
    do {                                                                                 \
        std::printf("kind %d term %d cm %#x p %d: ", kind, term, cm, p);                 \
        std::printf(__VA_ARGS__);                                                        \
        std::printf("\n");                                                               \
        return 1;                                                                        \
    } while (0)

int main()
{
    long checks = 0;
    for (int kind = 0; kind < 2; ++kind)
        for (int term = 1; term <= 3; ++term) {
            const int dim = term + 4, np = rule_points(dim), nax = 1 + 4 * dim, zd = dim - 1;
            uint32_t code[256];
            for (int p = 0; p < np; ++p) code[p] = point_variants(dim, p);
            for (unsigned cm = 1; cm < (1u << dim); ++cm)
                for (int p = 0; p < np; ++p) {
                    if (!split_point(cm, p, nax)) continue;
                    auto var = [&](int d) { return (int)((code[p] >> (3 * d)) & 7u); };
                    for (int d = 0; d < dim; ++d, ++checks)
                        if (!split_variant(cm, d, var(d))) FAIL("slot %d/%d not filled", d, var(d));
                    for (int f = 0; f < ucache_nf(term); ++f, ++checks) {
                        const int dl = ucache_fun(kind, term, f, 0), dm = ucache_fun(kind, term, f, 1);
                        const int vl = var(dl), vm = var(dm), vz = var(zd);
                        if ((vl != 0) + (vm != 0) + (vz != 0) > 1 || !split_variant(cm, dl, vl) ||
                            !split_variant(cm, dm, vm) || !split_variant(cm, zd, vz))
                            FAIL("u_NFW combination %d (%d,%d,%d) not computed", f, vl, vm, vz);
                        if (!pair_computed(cm, dm, zd, vm, vz))
                            FAIL("(mass, z) pair of combination %d not computed", f);
                    }
                    for (int f = 0; f < u3_nfun(term); ++f, ++checks) {
                        const int q = first_of(code, p, ~u3_drop(kind, term, f));
                        if (!split_point(cm, q, nax)) FAIL("k3 projection %d (first point %d)", f, q);
                        const int md = u3_mass(kind, term, f);
                        if (!pair_computed(cm, md, zd, (code[q] >> (3 * md)) & 7u, (code[q] >> (3 * zd)) & 7u))
                            FAIL("(mass, z) pair of k3 projection %d not computed", f);
                    }
                    for (int a = 0; a < aux_nfun(term); ++a, ++checks) {
                        const int q = first_of(code, p, aux_keep(term, a));
                        if (!split_point(cm, q, nax)) FAIL("auxiliary projection %d (first point %d)", a, q);
                    }
                    if (term == 1 && !pair_computed(cm, 3, zd, var(3), var(zd)))
                        FAIL("(mass, z) pair of the 1-halo point not computed");
                    ++checks;
                }
        }
    std::printf("ok %ld\n", checks);
    return 0;
}
