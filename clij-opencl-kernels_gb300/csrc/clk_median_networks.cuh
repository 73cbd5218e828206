// clk_median_networks.cuh - GENERATED by gen_median_networks.py; do not edit.
// Pruned odd-even merge networks for the fast median kernels.  Each
// function works in place on w[]; the comment under it lists the wires
// that hold the consumed ranks afterwards.
#pragma once
#ifndef CLK_NET_FN
#define CLK_NET_FN __device__ __forceinline__
#endif
#ifndef CLK_NET_CONST
#define CLK_NET_CONST __device__ constexpr
#endif

// w[0..2] -> ranks in order [0, 1, 2]
// 6 min/max operations
template <class V> CLK_NET_FN void net_sort3_raw(V (&w)[3]) {
  { const V t = vmin(w[0], w[1]); w[1] = vmax(w[0], w[1]); w[0] = t; }
  { const V t = vmin(w[0], w[2]); w[2] = vmax(w[0], w[2]); w[0] = t; }
  { const V t = vmin(w[1], w[2]); w[2] = vmax(w[1], w[2]); w[1] = t; }
}
CLK_NET_CONST int net_sort3_out[3] = {0, 1, 2};

// three sorted triples w[0..2], w[3..5], w[6..8] -> sorted 9
// 36 min/max operations
template <class V> CLK_NET_FN void net_merge333_raw(V (&w)[9]) {
  { const V t = vmin(w[0], w[3]); w[3] = vmax(w[0], w[3]); w[0] = t; }
  { const V t = vmin(w[2], w[5]); w[5] = vmax(w[2], w[5]); w[2] = t; }
  { const V t = vmin(w[2], w[3]); w[3] = vmax(w[2], w[3]); w[2] = t; }
  { const V t = vmin(w[1], w[4]); w[4] = vmax(w[1], w[4]); w[1] = t; }
  { const V t = vmin(w[1], w[2]); w[2] = vmax(w[1], w[2]); w[1] = t; }
  { const V t = vmin(w[4], w[3]); w[3] = vmax(w[4], w[3]); w[4] = t; }
  { const V t = vmin(w[0], w[6]); w[6] = vmax(w[0], w[6]); w[0] = t; }
  { const V t = vmin(w[3], w[6]); w[6] = vmax(w[3], w[6]); w[3] = t; }
  { const V t = vmin(w[2], w[8]); w[8] = vmax(w[2], w[8]); w[2] = t; }
  { const V t = vmin(w[2], w[3]); w[3] = vmax(w[2], w[3]); w[2] = t; }
  { const V t = vmin(w[8], w[6]); w[6] = vmax(w[8], w[6]); w[8] = t; }
  { const V t = vmin(w[1], w[7]); w[7] = vmax(w[1], w[7]); w[1] = t; }
  { const V t = vmin(w[5], w[7]); w[7] = vmax(w[5], w[7]); w[5] = t; }
  { const V t = vmin(w[4], w[5]); w[5] = vmax(w[4], w[5]); w[4] = t; }
  { const V t = vmin(w[1], w[2]); w[2] = vmax(w[1], w[2]); w[1] = t; }
  { const V t = vmin(w[4], w[3]); w[3] = vmax(w[4], w[3]); w[4] = t; }
  { const V t = vmin(w[5], w[8]); w[8] = vmax(w[5], w[8]); w[5] = t; }
  { const V t = vmin(w[7], w[6]); w[6] = vmax(w[7], w[6]); w[7] = t; }
}
CLK_NET_CONST int net_merge333_out[9] = {0, 1, 2, 4, 3, 5, 8, 7, 6};

// sorted triples w[0..2], w[3..5] -> sorted 6
// 12 min/max operations
template <class V> CLK_NET_FN void net_merge33_raw(V (&w)[6]) {
  { const V t = vmin(w[0], w[3]); w[3] = vmax(w[0], w[3]); w[0] = t; }
  { const V t = vmin(w[2], w[5]); w[5] = vmax(w[2], w[5]); w[2] = t; }
  { const V t = vmin(w[2], w[3]); w[3] = vmax(w[2], w[3]); w[2] = t; }
  { const V t = vmin(w[1], w[4]); w[4] = vmax(w[1], w[4]); w[1] = t; }
  { const V t = vmin(w[1], w[2]); w[2] = vmax(w[1], w[2]); w[1] = t; }
  { const V t = vmin(w[4], w[3]); w[3] = vmax(w[4], w[3]); w[4] = t; }
}
CLK_NET_CONST int net_merge33_out[6] = {0, 1, 2, 4, 3, 5};

// sorted 6 w[0..5] and sorted triple w[6..8] -> sorted 9
// 24 min/max operations
template <class V> CLK_NET_FN void net_merge63_raw(V (&w)[9]) {
  { const V t = vmin(w[0], w[6]); w[6] = vmax(w[0], w[6]); w[0] = t; }
  { const V t = vmin(w[4], w[6]); w[6] = vmax(w[4], w[6]); w[4] = t; }
  { const V t = vmin(w[2], w[8]); w[8] = vmax(w[2], w[8]); w[2] = t; }
  { const V t = vmin(w[2], w[4]); w[4] = vmax(w[2], w[4]); w[2] = t; }
  { const V t = vmin(w[8], w[6]); w[6] = vmax(w[8], w[6]); w[8] = t; }
  { const V t = vmin(w[1], w[7]); w[7] = vmax(w[1], w[7]); w[1] = t; }
  { const V t = vmin(w[5], w[7]); w[7] = vmax(w[5], w[7]); w[5] = t; }
  { const V t = vmin(w[3], w[5]); w[5] = vmax(w[3], w[5]); w[3] = t; }
  { const V t = vmin(w[1], w[2]); w[2] = vmax(w[1], w[2]); w[1] = t; }
  { const V t = vmin(w[3], w[4]); w[4] = vmax(w[3], w[4]); w[3] = t; }
  { const V t = vmin(w[5], w[8]); w[8] = vmax(w[5], w[8]); w[5] = t; }
  { const V t = vmin(w[7], w[6]); w[6] = vmax(w[7], w[6]); w[7] = t; }
}
CLK_NET_CONST int net_merge63_out[9] = {0, 1, 2, 3, 4, 5, 8, 7, 6};

// sorted 9s w[0..8], w[9..17] -> ranks 4..13
// 48 min/max operations
template <class V> CLK_NET_FN void net_merge99_mid_raw(V (&w)[18]) {
  w[9] = vmax(w[0], w[9]);
  w[8] = vmin(w[8], w[17]);
  { const V t = vmin(w[8], w[9]); w[9] = vmax(w[8], w[9]); w[8] = t; }
  { const V t = vmin(w[4], w[13]); w[13] = vmax(w[4], w[13]); w[4] = t; }
  { const V t = vmin(w[4], w[8]); w[8] = vmax(w[4], w[8]); w[4] = t; }
  { const V t = vmin(w[13], w[9]); w[9] = vmax(w[13], w[9]); w[13] = t; }
  { const V t = vmin(w[2], w[11]); w[11] = vmax(w[2], w[11]); w[2] = t; }
  { const V t = vmin(w[6], w[15]); w[15] = vmax(w[6], w[15]); w[6] = t; }
  { const V t = vmin(w[6], w[11]); w[11] = vmax(w[6], w[11]); w[6] = t; }
  w[4] = vmax(w[2], w[4]);
  { const V t = vmin(w[6], w[8]); w[8] = vmax(w[6], w[8]); w[6] = t; }
  { const V t = vmin(w[11], w[13]); w[13] = vmax(w[11], w[13]); w[11] = t; }
  w[15] = vmin(w[15], w[9]);
  w[10] = vmax(w[1], w[10]);
  { const V t = vmin(w[5], w[14]); w[14] = vmax(w[5], w[14]); w[5] = t; }
  { const V t = vmin(w[5], w[10]); w[10] = vmax(w[5], w[10]); w[5] = t; }
  { const V t = vmin(w[3], w[12]); w[12] = vmax(w[3], w[12]); w[3] = t; }
  w[7] = vmin(w[7], w[16]);
  { const V t = vmin(w[7], w[12]); w[12] = vmax(w[7], w[12]); w[7] = t; }
  { const V t = vmin(w[3], w[5]); w[5] = vmax(w[3], w[5]); w[3] = t; }
  { const V t = vmin(w[7], w[10]); w[10] = vmax(w[7], w[10]); w[7] = t; }
  { const V t = vmin(w[12], w[14]); w[14] = vmax(w[12], w[14]); w[12] = t; }
  w[4] = vmax(w[3], w[4]);
  { const V t = vmin(w[5], w[6]); w[6] = vmax(w[5], w[6]); w[5] = t; }
  { const V t = vmin(w[7], w[8]); w[8] = vmax(w[7], w[8]); w[7] = t; }
  { const V t = vmin(w[10], w[11]); w[11] = vmax(w[10], w[11]); w[10] = t; }
  { const V t = vmin(w[12], w[13]); w[13] = vmax(w[12], w[13]); w[12] = t; }
  w[14] = vmin(w[14], w[15]);
}
CLK_NET_CONST int net_merge99_mid_out[10] = {4, 5, 6, 7, 8, 10, 11, 12, 13, 14};

// sorted 10 w[0..9] U sorted 9 w[10..18] -> rank 9
// 18 min/max operations
template <class V> CLK_NET_FN void net_box27_final_raw(V (&w)[19]) {
  w[10] = vmax(w[0], w[10]);
  w[8] = vmin(w[8], w[18]);
  w[10] = vmax(w[8], w[10]);
  w[14] = vmax(w[4], w[14]);
  w[14] = vmin(w[14], w[10]);
  w[12] = vmax(w[2], w[12]);
  w[6] = vmin(w[6], w[16]);
  w[12] = vmax(w[6], w[12]);
  w[12] = vmin(w[12], w[14]);
  w[11] = vmax(w[1], w[11]);
  w[9] = vmin(w[9], w[11]);
  w[5] = vmin(w[5], w[15]);
  w[9] = vmax(w[5], w[9]);
  w[13] = vmax(w[3], w[13]);
  w[7] = vmin(w[7], w[17]);
  w[7] = vmin(w[7], w[13]);
  w[9] = vmax(w[7], w[9]);
  w[9] = vmin(w[9], w[12]);
}
CLK_NET_CONST int net_box27_final_out[1] = {9};

// sorted 9 x3 + 4 + 2 singles -> rank 16
// 146 min/max operations
template <class V> CLK_NET_FN void net_sphere33_final_raw(V (&w)[33]) {
  { const V t = vmin(w[0], w[9]); w[9] = vmax(w[0], w[9]); w[0] = t; }
  { const V t = vmin(w[8], w[17]); w[17] = vmax(w[8], w[17]); w[8] = t; }
  { const V t = vmin(w[8], w[9]); w[9] = vmax(w[8], w[9]); w[8] = t; }
  { const V t = vmin(w[4], w[13]); w[13] = vmax(w[4], w[13]); w[4] = t; }
  { const V t = vmin(w[4], w[8]); w[8] = vmax(w[4], w[8]); w[4] = t; }
  { const V t = vmin(w[13], w[9]); w[9] = vmax(w[13], w[9]); w[13] = t; }
  { const V t = vmin(w[2], w[11]); w[11] = vmax(w[2], w[11]); w[2] = t; }
  { const V t = vmin(w[6], w[15]); w[15] = vmax(w[6], w[15]); w[6] = t; }
  { const V t = vmin(w[6], w[11]); w[11] = vmax(w[6], w[11]); w[6] = t; }
  { const V t = vmin(w[2], w[4]); w[4] = vmax(w[2], w[4]); w[2] = t; }
  { const V t = vmin(w[6], w[8]); w[8] = vmax(w[6], w[8]); w[6] = t; }
  { const V t = vmin(w[11], w[13]); w[13] = vmax(w[11], w[13]); w[11] = t; }
  { const V t = vmin(w[15], w[9]); w[9] = vmax(w[15], w[9]); w[15] = t; }
  { const V t = vmin(w[1], w[10]); w[10] = vmax(w[1], w[10]); w[1] = t; }
  { const V t = vmin(w[5], w[14]); w[14] = vmax(w[5], w[14]); w[5] = t; }
  { const V t = vmin(w[5], w[10]); w[10] = vmax(w[5], w[10]); w[5] = t; }
  { const V t = vmin(w[3], w[12]); w[12] = vmax(w[3], w[12]); w[3] = t; }
  { const V t = vmin(w[7], w[16]); w[16] = vmax(w[7], w[16]); w[7] = t; }
  { const V t = vmin(w[7], w[12]); w[12] = vmax(w[7], w[12]); w[7] = t; }
  { const V t = vmin(w[3], w[5]); w[5] = vmax(w[3], w[5]); w[3] = t; }
  { const V t = vmin(w[7], w[10]); w[10] = vmax(w[7], w[10]); w[7] = t; }
  { const V t = vmin(w[12], w[14]); w[14] = vmax(w[12], w[14]); w[12] = t; }
  { const V t = vmin(w[1], w[2]); w[2] = vmax(w[1], w[2]); w[1] = t; }
  { const V t = vmin(w[3], w[4]); w[4] = vmax(w[3], w[4]); w[3] = t; }
  { const V t = vmin(w[5], w[6]); w[6] = vmax(w[5], w[6]); w[5] = t; }
  { const V t = vmin(w[7], w[8]); w[8] = vmax(w[7], w[8]); w[7] = t; }
  { const V t = vmin(w[10], w[11]); w[11] = vmax(w[10], w[11]); w[10] = t; }
  { const V t = vmin(w[12], w[13]); w[13] = vmax(w[12], w[13]); w[12] = t; }
  { const V t = vmin(w[14], w[15]); w[15] = vmax(w[14], w[15]); w[14] = t; }
  { const V t = vmin(w[16], w[9]); w[9] = vmax(w[16], w[9]); w[16] = t; }
  w[18] = vmax(w[0], w[18]);
  w[9] = vmin(w[9], w[18]);
  w[8] = vmin(w[8], w[26]);
  w[9] = vmax(w[8], w[9]);
  w[22] = vmax(w[4], w[22]);
  w[13] = vmin(w[13], w[22]);
  { const V t = vmin(w[13], w[9]); w[9] = vmax(w[13], w[9]); w[13] = t; }
  w[20] = vmax(w[2], w[20]);
  { const V t = vmin(w[11], w[20]); w[20] = vmax(w[11], w[20]); w[11] = t; }
  { const V t = vmin(w[6], w[24]); w[24] = vmax(w[6], w[24]); w[6] = t; }
  w[15] = vmin(w[15], w[24]);
  w[11] = vmax(w[6], w[11]);
  w[15] = vmin(w[15], w[20]);
  { const V t = vmin(w[11], w[13]); w[13] = vmax(w[11], w[13]); w[11] = t; }
  { const V t = vmin(w[15], w[9]); w[9] = vmax(w[15], w[9]); w[15] = t; }
  w[19] = vmax(w[1], w[19]);
  w[17] = vmin(w[17], w[19]);
  { const V t = vmin(w[10], w[17]); w[17] = vmax(w[10], w[17]); w[10] = t; }
  { const V t = vmin(w[5], w[23]); w[23] = vmax(w[5], w[23]); w[5] = t; }
  w[14] = vmin(w[14], w[23]);
  w[10] = vmax(w[5], w[10]);
  { const V t = vmin(w[14], w[17]); w[17] = vmax(w[14], w[17]); w[14] = t; }
  w[21] = vmax(w[3], w[21]);
  { const V t = vmin(w[12], w[21]); w[21] = vmax(w[12], w[21]); w[12] = t; }
  { const V t = vmin(w[7], w[25]); w[25] = vmax(w[7], w[25]); w[7] = t; }
  w[16] = vmin(w[16], w[25]);
  { const V t = vmin(w[7], w[12]); w[12] = vmax(w[7], w[12]); w[7] = t; }
  w[16] = vmin(w[16], w[21]);
  w[10] = vmax(w[7], w[10]);
  { const V t = vmin(w[12], w[14]); w[14] = vmax(w[12], w[14]); w[12] = t; }
  w[16] = vmin(w[16], w[17]);
  w[11] = vmax(w[10], w[11]);
  { const V t = vmin(w[12], w[13]); w[13] = vmax(w[12], w[13]); w[12] = t; }
  { const V t = vmin(w[14], w[15]); w[15] = vmax(w[14], w[15]); w[14] = t; }
  { const V t = vmin(w[16], w[9]); w[9] = vmax(w[16], w[9]); w[16] = t; }
  { const V t = vmin(w[27], w[28]); w[28] = vmax(w[27], w[28]); w[27] = t; }
  { const V t = vmin(w[29], w[30]); w[30] = vmax(w[29], w[30]); w[29] = t; }
  { const V t = vmin(w[27], w[29]); w[29] = vmax(w[27], w[29]); w[27] = t; }
  { const V t = vmin(w[28], w[30]); w[30] = vmax(w[28], w[30]); w[28] = t; }
  { const V t = vmin(w[28], w[29]); w[29] = vmax(w[28], w[29]); w[28] = t; }
  { const V t = vmin(w[31], w[32]); w[32] = vmax(w[31], w[32]); w[31] = t; }
  { const V t = vmin(w[27], w[31]); w[31] = vmax(w[27], w[31]); w[27] = t; }
  { const V t = vmin(w[29], w[31]); w[31] = vmax(w[29], w[31]); w[29] = t; }
  { const V t = vmin(w[28], w[32]); w[32] = vmax(w[28], w[32]); w[28] = t; }
  { const V t = vmin(w[30], w[32]); w[32] = vmax(w[30], w[32]); w[30] = t; }
  { const V t = vmin(w[28], w[29]); w[29] = vmax(w[28], w[29]); w[28] = t; }
  { const V t = vmin(w[30], w[31]); w[31] = vmax(w[30], w[31]); w[30] = t; }
  w[16] = vmax(w[27], w[16]);
  w[15] = vmax(w[28], w[15]);
  w[14] = vmax(w[29], w[14]);
  w[13] = vmax(w[30], w[13]);
  w[12] = vmax(w[31], w[12]);
  w[11] = vmax(w[32], w[11]);
  w[9] = vmin(w[9], w[16]);
  w[9] = vmin(w[9], w[15]);
  w[9] = vmin(w[9], w[14]);
  w[9] = vmin(w[9], w[13]);
  w[9] = vmin(w[9], w[12]);
  w[9] = vmin(w[9], w[11]);
}
CLK_NET_CONST int net_sphere33_final_out[1] = {9};

// sorted 9s w[0..8], w[9..17] -> ranks 1..16
// 58 min/max operations
template <class V> CLK_NET_FN void net_merge99_r1_16_raw(V (&w)[18]) {
  w[9] = vmax(w[0], w[9]);
  w[8] = vmin(w[8], w[17]);
  { const V t = vmin(w[8], w[9]); w[9] = vmax(w[8], w[9]); w[8] = t; }
  { const V t = vmin(w[4], w[13]); w[13] = vmax(w[4], w[13]); w[4] = t; }
  { const V t = vmin(w[4], w[8]); w[8] = vmax(w[4], w[8]); w[4] = t; }
  { const V t = vmin(w[13], w[9]); w[9] = vmax(w[13], w[9]); w[13] = t; }
  { const V t = vmin(w[2], w[11]); w[11] = vmax(w[2], w[11]); w[2] = t; }
  { const V t = vmin(w[6], w[15]); w[15] = vmax(w[6], w[15]); w[6] = t; }
  { const V t = vmin(w[6], w[11]); w[11] = vmax(w[6], w[11]); w[6] = t; }
  { const V t = vmin(w[2], w[4]); w[4] = vmax(w[2], w[4]); w[2] = t; }
  { const V t = vmin(w[6], w[8]); w[8] = vmax(w[6], w[8]); w[6] = t; }
  { const V t = vmin(w[11], w[13]); w[13] = vmax(w[11], w[13]); w[11] = t; }
  { const V t = vmin(w[15], w[9]); w[9] = vmax(w[15], w[9]); w[15] = t; }
  { const V t = vmin(w[1], w[10]); w[10] = vmax(w[1], w[10]); w[1] = t; }
  { const V t = vmin(w[5], w[14]); w[14] = vmax(w[5], w[14]); w[5] = t; }
  { const V t = vmin(w[5], w[10]); w[10] = vmax(w[5], w[10]); w[5] = t; }
  { const V t = vmin(w[3], w[12]); w[12] = vmax(w[3], w[12]); w[3] = t; }
  { const V t = vmin(w[7], w[16]); w[16] = vmax(w[7], w[16]); w[7] = t; }
  { const V t = vmin(w[7], w[12]); w[12] = vmax(w[7], w[12]); w[7] = t; }
  { const V t = vmin(w[3], w[5]); w[5] = vmax(w[3], w[5]); w[3] = t; }
  { const V t = vmin(w[7], w[10]); w[10] = vmax(w[7], w[10]); w[7] = t; }
  { const V t = vmin(w[12], w[14]); w[14] = vmax(w[12], w[14]); w[12] = t; }
  { const V t = vmin(w[1], w[2]); w[2] = vmax(w[1], w[2]); w[1] = t; }
  { const V t = vmin(w[3], w[4]); w[4] = vmax(w[3], w[4]); w[3] = t; }
  { const V t = vmin(w[5], w[6]); w[6] = vmax(w[5], w[6]); w[5] = t; }
  { const V t = vmin(w[7], w[8]); w[8] = vmax(w[7], w[8]); w[7] = t; }
  { const V t = vmin(w[10], w[11]); w[11] = vmax(w[10], w[11]); w[10] = t; }
  { const V t = vmin(w[12], w[13]); w[13] = vmax(w[12], w[13]); w[12] = t; }
  { const V t = vmin(w[14], w[15]); w[15] = vmax(w[14], w[15]); w[14] = t; }
  { const V t = vmin(w[16], w[9]); w[9] = vmax(w[16], w[9]); w[16] = t; }
}
CLK_NET_CONST int net_merge99_r1_16_out[16] = {1, 2, 3, 4, 5, 6, 7, 8, 10, 11, 12, 13, 14, 15, 16, 9};

// sorted 16 w[0..15] U sorted 9 w[16..24] U 6 singles -> rank 15
// 84 min/max operations
template <class V> CLK_NET_FN void net_sphere33_pair_final_raw(V (&w)[31]) {
  w[16] = vmax(w[0], w[16]);
  w[8] = vmin(w[8], w[24]);
  w[16] = vmax(w[8], w[16]);
  w[20] = vmax(w[4], w[20]);
  w[12] = vmin(w[12], w[20]);
  { const V t = vmin(w[12], w[16]); w[16] = vmax(w[12], w[16]); w[12] = t; }
  w[18] = vmax(w[2], w[18]);
  { const V t = vmin(w[10], w[18]); w[18] = vmax(w[10], w[18]); w[10] = t; }
  { const V t = vmin(w[6], w[22]); w[22] = vmax(w[6], w[22]); w[6] = t; }
  w[14] = vmin(w[14], w[22]);
  w[10] = vmax(w[6], w[10]);
  w[14] = vmin(w[14], w[18]);
  { const V t = vmin(w[10], w[12]); w[12] = vmax(w[10], w[12]); w[10] = t; }
  { const V t = vmin(w[14], w[16]); w[16] = vmax(w[14], w[16]); w[14] = t; }
  w[17] = vmax(w[1], w[17]);
  { const V t = vmin(w[9], w[17]); w[17] = vmax(w[9], w[17]); w[9] = t; }
  { const V t = vmin(w[5], w[21]); w[21] = vmax(w[5], w[21]); w[5] = t; }
  w[13] = vmin(w[13], w[21]);
  w[9] = vmax(w[5], w[9]);
  { const V t = vmin(w[13], w[17]); w[17] = vmax(w[13], w[17]); w[13] = t; }
  w[19] = vmax(w[3], w[19]);
  { const V t = vmin(w[11], w[19]); w[19] = vmax(w[11], w[19]); w[11] = t; }
  { const V t = vmin(w[7], w[23]); w[23] = vmax(w[7], w[23]); w[7] = t; }
  w[15] = vmin(w[15], w[23]);
  { const V t = vmin(w[7], w[11]); w[11] = vmax(w[7], w[11]); w[7] = t; }
  w[15] = vmin(w[15], w[19]);
  w[9] = vmax(w[7], w[9]);
  { const V t = vmin(w[11], w[13]); w[13] = vmax(w[11], w[13]); w[11] = t; }
  w[15] = vmin(w[15], w[17]);
  { const V t = vmin(w[9], w[10]); w[10] = vmax(w[9], w[10]); w[9] = t; }
  { const V t = vmin(w[11], w[12]); w[12] = vmax(w[11], w[12]); w[11] = t; }
  { const V t = vmin(w[13], w[14]); w[14] = vmax(w[13], w[14]); w[13] = t; }
  w[15] = vmin(w[15], w[16]);
  { const V t = vmin(w[25], w[26]); w[26] = vmax(w[25], w[26]); w[25] = t; }
  { const V t = vmin(w[27], w[28]); w[28] = vmax(w[27], w[28]); w[27] = t; }
  { const V t = vmin(w[25], w[27]); w[27] = vmax(w[25], w[27]); w[25] = t; }
  { const V t = vmin(w[26], w[28]); w[28] = vmax(w[26], w[28]); w[26] = t; }
  { const V t = vmin(w[26], w[27]); w[27] = vmax(w[26], w[27]); w[26] = t; }
  { const V t = vmin(w[29], w[30]); w[30] = vmax(w[29], w[30]); w[29] = t; }
  { const V t = vmin(w[25], w[29]); w[29] = vmax(w[25], w[29]); w[25] = t; }
  { const V t = vmin(w[27], w[29]); w[29] = vmax(w[27], w[29]); w[27] = t; }
  { const V t = vmin(w[26], w[30]); w[30] = vmax(w[26], w[30]); w[26] = t; }
  { const V t = vmin(w[28], w[30]); w[30] = vmax(w[28], w[30]); w[28] = t; }
  { const V t = vmin(w[26], w[27]); w[27] = vmax(w[26], w[27]); w[26] = t; }
  { const V t = vmin(w[28], w[29]); w[29] = vmax(w[28], w[29]); w[28] = t; }
  w[14] = vmax(w[25], w[14]);
  w[13] = vmax(w[26], w[13]);
  w[12] = vmax(w[27], w[12]);
  w[11] = vmax(w[28], w[11]);
  w[10] = vmax(w[29], w[10]);
  w[9] = vmax(w[30], w[9]);
  w[15] = vmin(w[15], w[14]);
  w[15] = vmin(w[15], w[13]);
  w[15] = vmin(w[15], w[12]);
  w[15] = vmin(w[15], w[11]);
  w[15] = vmin(w[15], w[10]);
  w[15] = vmin(w[15], w[9]);
}
CLK_NET_CONST int net_sphere33_pair_final_out[1] = {15};

// three sorted triples -> rank 4
// 20 min/max operations
template <class V> CLK_NET_FN void net_med9_raw(V (&w)[9]) {
  { const V t = vmin(w[0], w[3]); w[3] = vmax(w[0], w[3]); w[0] = t; }
  { const V t = vmin(w[2], w[5]); w[5] = vmax(w[2], w[5]); w[2] = t; }
  { const V t = vmin(w[2], w[3]); w[3] = vmax(w[2], w[3]); w[2] = t; }
  { const V t = vmin(w[1], w[4]); w[4] = vmax(w[1], w[4]); w[1] = t; }
  { const V t = vmin(w[1], w[2]); w[2] = vmax(w[1], w[2]); w[1] = t; }
  { const V t = vmin(w[4], w[3]); w[3] = vmax(w[4], w[3]); w[4] = t; }
  w[6] = vmax(w[0], w[6]);
  w[3] = vmin(w[3], w[6]);
  w[2] = vmin(w[2], w[8]);
  w[3] = vmax(w[2], w[3]);
  w[7] = vmax(w[1], w[7]);
  w[5] = vmin(w[5], w[7]);
  w[4] = vmin(w[4], w[5]);
  w[3] = vmax(w[4], w[3]);
}
CLK_NET_CONST int net_med9_out[1] = {3};
