// Reads a FASTA / FASTQ file through the C++ front end (read_sequences) and prints, per record,
// "name<TAB>sequence<TAB>quality" ("-" for an empty field); then the 2-bit words of all
// sequences and the count of non-ACGT bytes.  Host code only: runs without a GPU.
#include <iostream>

#include "pairwise_aligner_gb300.hpp"

namespace aligner = seqan::pairwise_aligner_gb300;

int main(int argc, char **argv)
{
    if (argc != 2) return 2;
    try {
        auto f = aligner::read_sequences(argv[1]);
        for (size_t k = 0; k < f.size(); ++k) {
            const auto seq = f.sequence(k);
            std::string qual = f.qualities.empty() ? std::string{} : f.qualities.substr(f.offsets[k], seq.size());
            std::cout << f.names[k] << '\t' << (seq.empty() ? std::string{"-"} : std::string{seq}) << '\t'
                      << (qual.empty() ? std::string{"-"} : qual) << '\n';
        }
        uint64_t bad = 0;
        for (uint32_t w : aligner::pack_2bit(f.sequences, &bad)) std::cout << w << ' ';
        std::cout << '\n' << bad << '\n';
    } catch (std::exception const &e) {
        std::cout << "error " << e.what() << '\n';
        return 1;
    }
    return 0;
}
