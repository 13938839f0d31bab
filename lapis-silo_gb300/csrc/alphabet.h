// Symbol alphabets of the sequence columns.
//
// Nucleotide: 16 IUPAC symbols, missing symbol N, valid mutation symbols {-,A,C,G,T}
//   (reference: src/rhydb/common/nucleotide_symbols.h:20-106).
// Amino acid: 28 symbols, missing symbol X, 24 valid mutation symbols
//   (reference: src/rhydb/common/aa_symbols.h:23-118).
// AMBIGUITY_SYMBOLS[s] = { y : CODES_FOR[s] is a subset of CODES_FOR[y] }
//   (reference: src/rhydb/common/nucleotide_symbols.cpp:11-72, aa_symbols.cpp).
// Symbol sets are bit masks (bit i = symbol with enum value i); both alphabets fit in 32 bits.
#pragma once

#include <cstdint>
#include <string>

namespace rhygpu {

enum class SymKind : uint8_t { NUC = 0, AA = 1 };

struct Alphabet {
   SymKind kind;
   uint32_t count;           // number of symbols
   uint8_t missing;          // N / X
   const char* chars;        // symbol -> char (upper case)
   uint32_t valid_mask;      // VALID_MUTATION_SYMBOLS
   uint32_t all_mask;        // every symbol
   uint32_t codes_for[32];   // CODES_FOR as masks
   uint32_t ambiguity[32];   // AMBIGUITY_SYMBOLS as masks
   int8_t char_to_sym[256];  // -1 = illegal character

   int sym(char c) const { return char_to_sym[static_cast<uint8_t>(c)]; }
};

const Alphabet& nucleotide();
const Alphabet& amino_acid();
inline const Alphabet& alphabet(SymKind k) { return k == SymKind::NUC ? nucleotide() : amino_acid(); }

// Standard genetic code translation of one codon (three nucleotide chars, upper case).
// Codons containing N or an ambiguity code translate to X; "---" translates to '-', a codon with
// one or two gaps translates to X.
char translate_codon(char a, char b, char c);

}  // namespace rhygpu
