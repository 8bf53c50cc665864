// Sequence generator of the reference's SIMD differential tests, restated.
//
// The reference's test fixture (test/unit/affine/alignment_simd_test_template.hpp:115-181)
// seeds std::mt19937 with 42, draws every sequence-1 length and symbols first,
// then every sequence-2, using std::uniform_int_distribution<size_t> for the
// length in [min, max] and for the symbol index into "ACGT".  This program
// reproduces those draws with the same standard-library engine and
// distributions so that tests/golden/ holds exactly the pairs the reference's
// own tests align.  The substitution-matrix tests draw from the matrix's symbol
// list instead (matrix_model::symbol_list, same file :62-77).
// Usage: gen_reference_sequences SEED COUNT MIN MAX [SYMBOLS]   (default ACGT)
// Output: COUNT lines of sequence 1, then COUNT lines of sequence 2.
#include <cstdio>
#include <cstdlib>
#include <random>
#include <string>
#include <vector>

int main(int argc, char **argv)
{
    if (argc != 5 && argc != 6) {
        std::fprintf(stderr, "usage: %s SEED COUNT MIN MAX [SYMBOLS]\n", argv[0]);
        return 2;
    }
    unsigned seed = static_cast<unsigned>(std::strtoul(argv[1], nullptr, 10));
    std::size_t count = std::strtoull(argv[2], nullptr, 10);
    std::size_t lo = std::strtoull(argv[3], nullptr, 10);
    std::size_t hi = std::strtoull(argv[4], nullptr, 10);
    const std::string symbols = argc == 6 ? argv[5] : "ACGT";
    if (symbols.empty()) return 2;

    std::mt19937 engine{seed};
    std::uniform_int_distribution<std::size_t> length_dist{lo, hi};
    std::uniform_int_distribution<std::size_t> symbol_dist{0, symbols.size() - 1};

    std::vector<std::string> out(2 * count);
    for (std::string &s : out) {
        s.resize(length_dist(engine));
        for (char &c : s) c = symbols[symbol_dist(engine)];
    }
    for (std::string const &s : out) std::printf("%s\n", s.c_str());
    return 0;
}
