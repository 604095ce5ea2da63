// TEST INFRASTRUCTURE: runs the reference's bitonic sort kernels
// (rtpslib/system/common/cl_src/bitonic.cl:54-258, compiled with
// LOCAL_SIZE_LIMIT=512 as BitonicSort.cpp:24 does) in the launch sequence of
// Bitonic<T>::Sort (rtpslib/system/common/BitonicSort.cpp:62-171) and
// System::bitonic_sort (rtpslib/system/System.cpp:407-455).
#define LOCAL_SIZE_LIMIT 512
#include "clshim.hpp"
#include "ref_api.h"
namespace rk_bit {
#include "cl_common/bitonic.cl"
}
#include <vector>

static unsigned next_pow2(unsigned x) {  // RTPSSettings.cpp:31-40 (nlpo2)
    x--;
    x |= x >> 1; x |= x >> 2; x |= x >> 4; x |= x >> 8; x |= x >> 16;
    return x + 1;
}

extern "C" void ref_bitonic_sort(int n, uint32_t* keys, uint32_t* idx) {
    if (n < 1) return;
    const unsigned L = next_pow2((unsigned)n);
    // Buffers of max_num entries filled with INT_MAX beyond num
    // (System.cpp:274-284); the local kernels always touch LOCAL_SIZE_LIMIT.
    const size_t cap = L < LOCAL_SIZE_LIMIT ? LOCAL_SIZE_LIMIT : L;
    std::vector<uint32_t> sk(cap, 0x7fffffffu), sv(cap, 0x7fffffffu), dk(cap, 0x7fffffffu), dv(cap, 0x7fffffffu);
    for (int i = 0; i < n; ++i) { sk[i] = keys[i]; sv[i] = idx[i]; }
    const unsigned dir = 1;
    if (L >= 2) {
        const size_t local = LOCAL_SIZE_LIMIT / 2;
        if (L <= LOCAL_SIZE_LIMIT) {
            clshim::launch_groups(round_up(L / 2, local), local, [&] {
                rk_bit::bitonicSortLocal(dk.data(), dv.data(), sk.data(), sv.data(), L, dir);
            });
        } else {
            clshim::launch_groups(round_up(L / 2, local), local, [&] {
                rk_bit::bitonicSortLocal1(dk.data(), dv.data(), sk.data(), sv.data());
            });
            for (unsigned size = 2 * LOCAL_SIZE_LIMIT; size <= L; size <<= 1) {
                for (unsigned stride = size / 2; stride > 0; stride >>= 1) {
                    if (stride >= LOCAL_SIZE_LIMIT) {
                        // Kernel::execute with no local size: every item is independent
                        clshim::launch_flat(L / 2, 1, [&] {
                            rk_bit::bitonicMergeGlobal(dk.data(), dv.data(), dk.data(), dv.data(), L, size, stride,
                                                       dir);
                        });
                    } else {
                        clshim::launch_groups(round_up(L / 2, local), local, [&] {
                            rk_bit::bitonicMergeLocal(dk.data(), dv.data(), dk.data(), dv.data(), L, stride, size,
                                                      dir);
                        });
                        break;
                    }
                }
            }
        }
    }
    // copyFromBuffer out -> in for num entries (System.cpp:451-452)
    for (int i = 0; i < n; ++i) { keys[i] = dk[i]; idx[i] = dv[i]; }
}
