// One translation unit per reference kernel file: compiled with -include ref_shim.hpp,
// -DREF_KERNEL_FILE="<path of the .cl>" and -DREF_KERNEL_NAME=<kernel function>.
// TEST INFRASTRUCTURE ONLY (see ref_shim.hpp).
#include REF_KERNEL_FILE

#define REF_CAT2(a, b) a##b
#define REF_CAT(a, b) REF_CAT2(a, b)

namespace {
typedef void (*RefItemFn)(const RefArgs&);

template <int G>
void ref_run_item(const RefArgs& a) {
    REF_KERNEL_NAME<G>(a.posX, a.posY, a.posZ, a.velX, a.velY, a.velZ, a.accX, a.accY, a.accZ,
                       a.step, a.blockCount, a.bodyCount, a.radius, a.maxDepth, a.bottom, a.mass,
                       a.child, a.start, a.sorted, a.error);
}

template <int... Gs>
constexpr std::array<RefItemFn, sizeof...(Gs)> ref_table(std::integer_sequence<int, Gs...>) {
    return {{&ref_run_item<Gs>...}};
}

const std::array<RefItemFn, NUM_WORK_GROUPS> kTable =
    ref_table(std::make_integer_sequence<int, NUM_WORK_GROUPS>());
}  // namespace

extern "C" void REF_CAT(ref_item_, REF_KERNEL_NAME)(int group, const RefArgs* a) { kTable[group](*a); }
