// clk_batch_max.cu - instantiations of the batched separable kernel
// (clk_batch.cuh) for maximum_separable: every batch pixel type, the XY radii of
// kBatchRadii and the generic-radius variant.
#include "clk_batch.cuh"

namespace clk {
namespace batch {

template <> const void* batch_sep_kernel_op<SEP_MAX>(int R, int dt) {
  auto pick = [&](auto r) -> const void* {
    constexpr int RR = decltype(r)::value;
    switch (dt) {
      case CLK_U8: return (const void*)k_batch_sep<SEP_MAX, RR, uint8_t>;
      case CLK_U16: return (const void*)k_batch_sep<SEP_MAX, RR, uint16_t>;
      case CLK_I16: return (const void*)k_batch_sep<SEP_MAX, RR, int16_t>;
      case CLK_F32: return (const void*)k_batch_sep<SEP_MAX, RR, float>;
    }
    return nullptr;
  };
  switch (R) {
    case 0: return pick(std::integral_constant<int, 0>{});
    case 2: return pick(std::integral_constant<int, 2>{});
    case 3: return pick(std::integral_constant<int, 3>{});
    case 4: return pick(std::integral_constant<int, 4>{});
    case 5: return pick(std::integral_constant<int, 5>{});
    case 6: return pick(std::integral_constant<int, 6>{});
  }
  return nullptr;
}

template <> const void* batch_sep2_kernel_op<SEP_MAX>(int R, int dt) {
  auto pick = [&](auto r) -> const void* {
    constexpr int RR = decltype(r)::value;
    switch (dt) {
      case CLK_U8: return (const void*)k_batch_sep2<SEP_MAX, RR, uint8_t>;
      case CLK_U16: return (const void*)k_batch_sep2<SEP_MAX, RR, uint16_t>;
      case CLK_I16: return (const void*)k_batch_sep2<SEP_MAX, RR, int16_t>;
      case CLK_F32: return (const void*)k_batch_sep2<SEP_MAX, RR, float>;
    }
    return nullptr;
  };
  switch (R) {
    case 2: return pick(std::integral_constant<int, 2>{});
    case 3: return pick(std::integral_constant<int, 3>{});
    case 4: return pick(std::integral_constant<int, 4>{});
    case 5: return pick(std::integral_constant<int, 5>{});
    case 6: return pick(std::integral_constant<int, 6>{});
  }
  return nullptr;
}

}  // namespace batch
}  // namespace clk
