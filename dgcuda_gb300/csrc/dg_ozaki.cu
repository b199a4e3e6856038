// dg_ozaki.cu -- host side of the tensor-core contractions: the f16 digit
// words and column exponents of the element kernel's four basis tables.
#include <cstring>
#include <vector>

#include "dg_internal.h"
#include "dg_tables_data.h"

#include "dg_ozaki.cuh"

namespace dg {
namespace oz {
namespace {

int host_bexp(double x) {
  unsigned long long b;
  std::memcpy(&b, &x, 8);
  return (int)((b >> 52) & 0x7FF);
}

long long host_fixed(double x, int m) {
  unsigned long long b;
  std::memcpy(&b, &x, 8);
  const int eb = (int)((b >> 52) & 0x7FF);
  const unsigned long long mant = (b & 0xFFFFFFFFFFFFFull) | (eb ? (1ull << 52) : 0ull);
  const int sh = m - (eb ? eb : 1);
  const unsigned long long X = sh < 64 ? (mant >> sh) : 0ull;
  const long long v = (b >> 63) ? -(long long)X : (long long)X;
  return v + (long long)kBias;
}

// f16 bit pattern of an integer in [-128, 127] (exact)
unsigned short half_of(int v) {
  if (v == 0) return 0;
  const unsigned short sign = v < 0 ? 0x8000 : 0;
  unsigned a = (unsigned)(v < 0 ? -v : v);
  int e = 0;
  while ((a >> (e + 1)) != 0) e++;
  const unsigned mant = (a << (10 - e)) & 0x3FF;
  return (unsigned short)(sign | ((e + 15) << 10) | mant);
}

// one table: T[kb][kslot][nslot] -> words and column exponents
void split_table(const double (*T)[16][16], int KB, uint2 *words, int *colexp) {
  for (int n = 0; n < 16; n++) {
    int M = 0;
    for (int kb = 0; kb < KB; kb++)
      for (int k = 0; k < 16; k++) M = M > host_bexp(T[kb][k][n]) ? M : host_bexp(T[kb][k][n]);
    colexp[n] = M ? M : 1023;  // an all-zero column: any exponent, digits are 0
  }
  auto digit = [&](int i, int kb, int k, int n) {
    const long long Y = host_fixed(T[kb][k][n], colexp[n]);
    return (int)((Y >> (8 * i)) & 255) - 128;
  };
  for (int i = 0; i < kDigits; i++)
    for (int kb = 0; kb < KB; kb++)
      for (int cg = 0; cg < 2; cg++)
        for (int lane = 0; lane < 32; lane++) {
          const int g = lane >> 2, t = lane & 3, n = cg * 8 + g;
          uint2 w;
          w.x = half_of(digit(i, kb, 2 * t, n)) | ((unsigned)half_of(digit(i, kb, 2 * t + 1, n)) << 16);
          w.y = half_of(digit(i, kb, 2 * t + 8, n)) |
                ((unsigned)half_of(digit(i, kb, 2 * t + 9, n)) << 16);
          words[((i * KB + kb) * 2 + cg) * 32 + lane] = w;
        }
}

int slot(int item) { return slot_of(item / 4, item % 4); }

}  // namespace

// the three tables as dense [K block][K slot][N slot] matrices of doubles:
// EVAL (1 block), PROJ (3), TRACE (1), in that order (5 x 16 x 16)
template <int P>
void dense_tables(const Tab<P> &tb, double (*T)[16][16]) {
  constexpr int NP = Tab<P>::NP, NQ = Tab<P>::NQ, N1 = Tab<P>::N1;
  std::memset(T, 0, sizeof(double) * 5 * 16 * 16);
  for (int q = 0; q < NQ; q++)
    for (int i = 0; i < NP; i++) {
      T[0][slot(i)][slot(q)] = tb.B[q][i];    // EVAL: u(q) = sum_i c_i B[q][i]
      T[1][slot(q)][slot(i)] = tb.GR[q][i];   // PROJ: sum_q GR g_q + GS h_q
      T[2][slot(q)][slot(i)] = tb.GS[q][i];
    }
  for (int f = 0; f < 3; f++)
    for (int j = 0; j < N1; j++)
      for (int i = 0; i < NP; i++) {
        T[3][slot(f * N1 + j)][slot(i)] = tb.E[f][j][i];  // PROJ: + sum_fj E F_fj
        T[4][slot(i)][slot(f * N1 + j)] = tb.E[f][j][i];  // TRACE: u_fj = sum_i E c_i
      }
}

template <int P>
void build_tabs(const Tab<P> &tb, Tabs *out, double *dense) {
  static double T[5][16][16];
  dense_tables<P>(tb, T);
  if (dense) std::memcpy(dense, T, sizeof T);
  std::memset(out, 0, sizeof *out);
  split_table(T, 1, out->w + word_off(kEval), out->colexp[kEval]);
  split_table(T + 1, 3, out->w + word_off(kProj), out->colexp[kProj]);
  split_table(T + 4, 1, out->w + word_off(kTrace), out->colexp[kTrace]);
}

}  // namespace oz

size_t oz_tabs_bytes() { return sizeof(oz::Tabs); }

bool oz_build_tabs(int p, const void *tabimg, void *out, double *dense) {
  oz::Tabs *o = static_cast<oz::Tabs *>(out);
  switch (p) {
    case 1: oz::build_tabs<1>(*static_cast<const Tab<1> *>(tabimg), o, dense); return true;
    case 2: oz::build_tabs<2>(*static_cast<const Tab<2> *>(tabimg), o, dense); return true;
    case 3: oz::build_tabs<3>(*static_cast<const Tab<3> *>(tabimg), o, dense); return true;
    case 4: oz::build_tabs<4>(*static_cast<const Tab<4> *>(tabimg), o, dense); return true;
    default: return false;
  }
}

}  // namespace dg

// the tensor-core table image of order p (1..4) built from the library's
// exact basis tables: 2240 uint2 digit words, then 3 x 16 int column
// exponents (and 16 ints of padding); bytes must be at least that size.
// dense (optional, 1280 doubles): the tables that were split, as dense
// [K block][K slot][N slot] matrices (EVAL, PROJ x 3, TRACE)
extern "C" dg_status dg_oz_table_image(int p, void *out, size_t bytes, double *dense) {
  if (p < 1 || p > 4 || !out) return dg::fail(DG_BAD_ARG, "order must be 1..4");
  if (bytes < sizeof(dg::oz::Tabs)) return dg::fail(DG_BAD_ARG, "buffer too small");
  std::vector<char> tab(dg::tab_bytes(p));
  dg::build_tab(p, DG_TABLES[p], tab.data());
  dg::oz_build_tabs(p, tab.data(), out, dense);
  return DG_OK;
}
