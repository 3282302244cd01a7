// One tcgen05.mma of kind::i8 (int8 x int8 -> int32 on the 5th-generation
// tensor cores).  Compiled only, never run: the test checks whether ptxas
// accepts the instruction for a target.
#include <cstdint>
__global__ void k_mma_i8(uint32_t tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                         uint32_t accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::i8 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate));
}
