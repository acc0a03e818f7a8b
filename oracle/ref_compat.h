/* Force-included (nvcc -include) when compiling the reference's own sources for the
 * distribution check. CUDA 13's Thrust no longer provides thrust::binary_function, which
 * the reference's parser derives a functor from (src/io/parser.cu:25-28); this restores
 * the empty base so the reference compiles unmodified. Test infrastructure only. */
#ifndef PROCELL_REF_COMPAT_H
#define PROCELL_REF_COMPAT_H
namespace thrust {
template <typename A, typename B, typename R>
struct binary_function {
  typedef A first_argument_type;
  typedef B second_argument_type;
  typedef R result_type;
};
}  // namespace thrust
#endif
