// Runs alignments through the C++20 front-end (include/pairwise_aligner_gb300.hpp)
// with the reference's rule nesting.  stdin: one case per line,
//   method open ext match mismatch first_column first_row last_column last_row seq1 seq2
// (method 0 global / 1 local, end-gap flags 0 penalised / 1 free, "-" = empty sequence).
// A line starting with "T" prints the global alignment (compute_alignments) as
//   "score begin1 begin2 end1 end2 cigar";
// a line starting with "M" scores with a substitution matrix (cfg::score_model_matrix):
//   M method open ext first_column first_row last_column last_row dim symbols s_0 .. s_{dim*dim-1} seq1 seq2
// stdout: "score end1 end2" per case, all cases of one configuration aligned in one bulk call.
#include <array>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "pairwise_aligner_gb300.hpp"

namespace aligner = seqan::pairwise_aligner_gb300;

// The reference's argument type: std::array<std::pair<symbol, std::array<score, D>>, D>.
template <size_t D>
void run_matrix(std::istringstream &in, int method, int open, int ext, int fc, int fr, int lc, int lr)
{
    std::string symbols, s1, s2;
    in >> symbols;
    std::array<std::pair<char, std::array<int, D>>, D> m{};
    for (size_t r = 0; r < D; ++r) {
        m[r].first = symbols.at(r);
        for (size_t k = 0; k < D; ++k) in >> m[r].second[k];
    }
    in >> s1 >> s2;
    if (s1 == "-") s1.clear();
    if (s2 == "-") s2.clear();
    using aligner::cfg::end_gap;
    auto e = [](int f) { return f ? end_gap::free : end_gap::penalised; };
    if (method == 1) {
        auto a = aligner::cfg::configure_aligner(
            aligner::cfg::score_model_matrix(aligner::cfg::method_local(aligner::cfg::gap_model_affine(open, ext)), m));
        auto r = a.compute(s1, s2);
        std::cout << r.score() << ' ' << r.end_position().first << ' ' << r.end_position().second << '\n';
    } else {
        auto a = aligner::cfg::configure_aligner(aligner::cfg::score_model_matrix(
            aligner::cfg::method_global(aligner::cfg::gap_model_affine(open, ext),
                                        aligner::cfg::leading_end_gap{e(fc), e(fr)},
                                        aligner::cfg::trailing_end_gap{e(lc), e(lr)}),
            m));
        auto r = a.compute(s1, s2);
        std::cout << r.score() << ' ' << r.end_position().first << ' ' << r.end_position().second << '\n';
    }
}

int main()
{
    std::string line;
    while (std::getline(std::cin, line)) {
        if (line.empty()) continue;
        std::istringstream in{line};
        if (line[0] == 'T') {                          // T match mismatch open ext seq1 seq2: global alignment
            std::string tag, a, b;
            int match, mismatch, open, ext;
            in >> tag >> match >> mismatch >> open >> ext >> a >> b;
            if (a == "-") a.clear();
            if (b == "-") b.clear();
            try {
                auto al = aligner::cfg::configure_aligner(aligner::cfg::score_model_unitary(
                    aligner::cfg::method_global(aligner::cfg::gap_model_affine(open, ext)), match, mismatch));
                std::vector<std::string> s1{a}, s2{b};
                auto r = al.compute_alignments(s1, s2).front();
                std::cout << r.score() << ' ' << r.begin_position().first << ' ' << r.begin_position().second << ' '
                          << r.end_position().first << ' ' << r.end_position().second << ' '
                          << (r.cigar().empty() ? "-" : r.cigar()) << '\n';
            } catch (std::exception const &ex) {
                std::cout << "error " << ex.what() << '\n';
            }
            continue;
        }
        if (line[0] == 'M') {
            std::string tag;
            int method, open, ext, fc, fr, lc, lr, dim;
            in >> tag >> method >> open >> ext >> fc >> fr >> lc >> lr >> dim;
            try {
                if (dim == 21) run_matrix<21>(in, method, open, ext, fc, fr, lc, lr);
                else if (dim == 27) run_matrix<27>(in, method, open, ext, fc, fr, lc, lr);
                else std::cout << "error unsupported dim\n";
            } catch (std::exception const &ex) {
                std::cout << "error " << ex.what() << '\n';
            }
            continue;
        }
        int method, open, ext, match, mismatch, fc, fr, lc, lr;
        std::string s1, s2;
        in >> method >> open >> ext >> match >> mismatch >> fc >> fr >> lc >> lr >> s1 >> s2;
        if (s1 == "-") s1.clear();
        if (s2 == "-") s2.clear();
        using aligner::cfg::end_gap;
        auto e = [](int f) { return f ? end_gap::free : end_gap::penalised; };
        std::vector<std::string> seqs1{s1}, seqs2{s2};
        try {
            if (method == 1) {
                auto a = aligner::cfg::configure_aligner(aligner::cfg::score_model_unitary(
                    aligner::cfg::method_local(aligner::cfg::gap_model_affine(open, ext)), match, mismatch));
                auto r = a.compute(seqs1, seqs2).front();
                std::cout << r.score() << ' ' << r.end_position().first << ' ' << r.end_position().second << '\n';
            } else {
                auto a = aligner::cfg::configure_aligner(aligner::cfg::score_model_unitary_simd_saturated(
                    aligner::cfg::method_global(aligner::cfg::gap_model_affine(open, ext),
                                                aligner::cfg::leading_end_gap{e(fc), e(fr)},
                                                aligner::cfg::trailing_end_gap{e(lc), e(lr)}),
                    match, mismatch));
                auto r = a.compute(s1, s2);
                std::cout << r.score() << ' ' << r.end_position().first << ' ' << r.end_position().second << '\n';
            }
        } catch (std::exception const &ex) {
            std::cout << "error " << ex.what() << '\n';
        }
    }
    return 0;
}
