// mrg8g_tables.h -- host-generated constants of the MRG8 recurrence.
//
// The generator state is s = (S[n-1], ..., S[n-8]) (newest first, as in
// original/mrg8.h:49) and one step is s' = A s with A the companion matrix:
// row 0 holds the coefficients a_1..a_8 (original/mrg8.cpp:16-18) and the
// sub-diagonal holds ones.  Everything here is computed on the host at load
// time; nothing is read from files.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define MRG8G_HDC __host__ __device__
#else
#define MRG8G_HDC
#endif

namespace mrg8g {

constexpr int kNumJump = 247;   // A^(2^i), i = 0..246 (jump_matrix.txt depth)

// Byte-window jump table of the device: jwin[w * 255 + j - 1] = A^(j 256^w)
// for byte position w = 0..7 and byte value j = 1..255, so a 64-bit jump is
// at most eight matrix-vector products (one per non-zero byte of the offset)
// instead of one per set bit.  jwin[0] = A (row 0 = the coefficients).
constexpr int kJumpBytes = 8;
constexpr int kJumpWinMats = kJumpBytes * 255;

// Lane layouts of the bulk kernels: a warp of 32 lanes, each lane writing V
// consecutive outputs per row, so consecutive rows of one lane are d = 32 V
// positions apart.  Supported V: 1, 2, 4 -> d = 32, 64, 128.
constexpr int kNumLayouts = 3;
MRG8G_HDC constexpr int layout_index(int V) { return V == 1 ? 0 : (V == 2 ? 1 : 2); }
MRG8G_HDC constexpr int layout_stride(int li) { return 32 << li; }
// Offsets (in u32 words) of each layout's window table inside one array.
MRG8G_HDC constexpr int win_offset(int li) { return li == 0 ? 0 : (li == 1 ? 32 * 64 : 96 * 64); }
constexpr int kWinWords = (32 + 64 + 128) * 64;

// Decimated recurrence.  The stride-d subsequence T_j = S[o + d j] of any
// MRG8 stream satisfies T_j = sum_k beta_k T_{j-k} (k = 1..8), where
// x^8 - sum beta_k x^(8-k) is the characteristic polynomial of A^d
// (Cayley-Hamilton).  For the kernels the coefficients are stored signed,
// c_k = beta_k or beta_k - p (|c_k| < 2^30), and the kernels keep the lagged
// values as x = S - 1 in [0, p-1] (`leap`); then
//     a = K1 + sum_k c_k x_{j-k}
// lies in [0, 2^64 - 1) and a == S_j - 1 (mod p), where K1 == sum_k c_k - 1
// (mod p) is the smallest such constant keeping a >= 0.  With the lagged
// values kept as s = S mod p instead (`leap_mod`, the fp64 ORIGINAL outputs), the
// same coefficients and K1 == 0 (mod p) give a == S_j (mod p).
struct LeapCoef {
    int32_t c[8];
    uint64_t K1;
};

struct HostTables {
    // jump[i][r*8+c] = A^(2^i)(r, c), row-major, canonical residues.
    uint32_t jump[kNumJump][64];
    // Byte windows (above), row-major like jump: 2040 matrices, 522,240 bytes.
    uint32_t jwin[kJumpWinMats][64];
    // Window tables, per layout li with stride d: win[off + (o*8 + j)*8 + c]
    // is column c of the row vector e_0^T A^(o + 1 + d j), o in [0, d),
    // j in [0, 8): S[B + o + d j] = win_row . s_B for a state s_B taken at
    // stream position B.
    uint32_t win[kWinWords];
    // Row-block steps of the layouts: dstep[li][j - 1] = A^(d j) for
    // d = layout_stride(li), j = 1..7 (the states at the starts of a warp's
    // first eight rows, from which its lanes form their windows).
    uint32_t dstep[kNumLayouts][7][64];
    LeapCoef leap[kNumLayouts];
    LeapCoef leap_mod[kNumLayouts];
};

// Built once (thread-safe) on first use.
const HostTables& host_tables();

// Row-major 8x8 product mod p, canonical entries.
void matmul_mod(const uint32_t* X, const uint32_t* Y, uint32_t* C);

// new_state = A^k state by per-bit matrix-vector products with the table
// (knl/mrg8.h:212-238).  Entries come back in [1, p] (0 only for an all-zero
// contribution), as bigDotProd does.
void jump_matvec(const uint32_t st[8], uint64_t k, uint32_t out[8]);

// Same over a 200-bit little-endian bit array (bits[i] != 0 -> set).
void jump_matvec_bits(const uint32_t st[8], const short bits[200], uint32_t out[8]);

// original/mrg8.cpp:104-176 exactly: J = product of A^(2^i) over the set bits
// formed with bigDotProd, then state <- J state.
void jump_exact_bits(const uint32_t st[8], const short bits[200], uint32_t out[8]);

// Sequential recurrence on the host for a handful of steps (state update of
// original/mrg8.cpp:197-222); outputs optional.
void step_host(uint32_t st[8], uint64_t n, uint32_t* out);

// seeding of original/mrg8.cpp:180-194.
void mcg64ni(uint32_t seed, uint32_t st[8]);

}  // namespace mrg8g
