#include "alphabet.h"

#include <cstring>

namespace rhygpu {
namespace {

void derive_ambiguity(Alphabet& a) {
   for (uint32_t s = 0; s < a.count; ++s) {
      uint32_t m = 0;
      for (uint32_t y = 0; y < a.count; ++y) {
         if ((a.codes_for[s] & a.codes_for[y]) == a.codes_for[s]) m |= 1u << y;
      }
      a.ambiguity[s] = m;
   }
}

void fill_char_map(Alphabet& a, const char* extra_upper_alias, int alias_sym) {
   std::memset(a.char_to_sym, -1, sizeof(a.char_to_sym));
   for (uint32_t s = 0; s < a.count; ++s) {
      const char c = a.chars[s];
      a.char_to_sym[static_cast<uint8_t>(c)] = static_cast<int8_t>(s);
      if (c >= 'A' && c <= 'Z') a.char_to_sym[static_cast<uint8_t>(c - 'A' + 'a')] = static_cast<int8_t>(s);
   }
   if (extra_upper_alias != nullptr) {
      for (const char* p = extra_upper_alias; *p; ++p) {
         a.char_to_sym[static_cast<uint8_t>(*p)] = static_cast<int8_t>(alias_sym);
      }
   }
}

Alphabet make_nuc() {
   Alphabet a{};
   a.kind = SymKind::NUC;
   a.count = 16;
   a.chars = "-ACGTRYSWKMBDHVN";
   a.missing = 15;
   // enum order: GAP A C G T R Y S W K M B D H V N
   enum { GAP, A, C, G, T, R, Y, S, W, K, M, B, D, H, V, N };
   auto bit = [](int s) { return 1u << s; };
   a.codes_for[GAP] = bit(GAP);
   a.codes_for[A] = bit(A);
   a.codes_for[C] = bit(C);
   a.codes_for[G] = bit(G);
   a.codes_for[T] = bit(T);
   a.codes_for[R] = bit(A) | bit(G);
   a.codes_for[Y] = bit(C) | bit(T);
   a.codes_for[S] = bit(G) | bit(C);
   a.codes_for[W] = bit(A) | bit(T);
   a.codes_for[K] = bit(G) | bit(T);
   a.codes_for[M] = bit(A) | bit(C);
   a.codes_for[B] = bit(C) | bit(G) | bit(T);
   a.codes_for[D] = bit(A) | bit(G) | bit(T);
   a.codes_for[H] = bit(A) | bit(C) | bit(T);
   a.codes_for[V] = bit(A) | bit(C) | bit(G);
   a.codes_for[N] = 0xFFFFu;
   a.all_mask = 0xFFFFu;
   a.valid_mask = bit(GAP) | bit(A) | bit(C) | bit(G) | bit(T);
   derive_ambiguity(a);
   fill_char_map(a, "Uu", T);
   return a;
}

Alphabet make_aa() {
   Alphabet a{};
   a.kind = SymKind::AA;
   a.count = 28;
   // enum order: GAP A C D E F G H I K L M N O P Q R S T U V W Y B J Z STOP X
   a.chars = "-ACDEFGHIKLMNOPQRSTUVWYBJZ*X";
   a.missing = 27;
   for (uint32_t s = 0; s < 28; ++s) a.codes_for[s] = 1u << s;
   const int D = 3, E = 4, I = 8, L = 10, N = 12, Q = 15;
   a.codes_for[23] = (1u << D) | (1u << N);  // B
   a.codes_for[24] = (1u << L) | (1u << I);  // J
   a.codes_for[25] = (1u << Q) | (1u << E);  // Z
   a.codes_for[27] = (1u << 28) - 1;         // X codes for every symbol
   a.all_mask = (1u << 28) - 1;
   a.valid_mask = ((1u << 23) - 1) | (1u << 26);  // GAP..Y and STOP
   derive_ambiguity(a);
   fill_char_map(a, nullptr, 0);
   return a;
}

int nuc_index(char c) {
   switch (c) {
      case 'T': return 0;
      case 'C': return 1;
      case 'A': return 2;
      case 'G': return 3;
      default: return -1;
   }
}

}  // namespace

const Alphabet& nucleotide() {
   static const Alphabet a = make_nuc();
   return a;
}

const Alphabet& amino_acid() {
   static const Alphabet a = make_aa();
   return a;
}

char translate_codon(char a, char b, char c) {
   // Standard code, bases ordered T, C, A, G: index = 16*i(a) + 4*i(b) + i(c).
   static const char* table = "FFLLSSSSYY**CC*WLLLLPPPPHHQQRRRRIIIMTTTTNNKKSSRRVVVVAAAADDEEGGGG";
   const int gaps = (a == '-') + (b == '-') + (c == '-');
   if (gaps == 3) return '-';
   if (gaps > 0) return 'X';
   const int ia = nuc_index(a), ib = nuc_index(b), ic = nuc_index(c);
   if (ia < 0 || ib < 0 || ic < 0) return 'X';
   return table[16 * ia + 4 * ib + ic];
}

}  // namespace rhygpu
