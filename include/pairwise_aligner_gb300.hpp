// pairwise_aligner_gb300.hpp -- header-only C++20 front-end of the GB300 DP.
//
// Keeps the configuration and call shape of the reference library so that its
// callers switch with a namespace alias:
//
//     namespace aligner = seqan::pairwise_aligner_gb300;   // was seqan::pairwise_aligner
//     auto a = aligner::cfg::configure_aligner(
//         aligner::cfg::method_global(
//             aligner::cfg::gap_model_affine(aligner::cfg::score_model_unitary_simd_saturated(4, -5), -10, -1),
//             aligner::cfg::leading_end_gap{}, aligner::cfg::trailing_end_gap{}));
//     for (auto const & r : a.compute(seqs1, seqs2)) r.score();
//
// Reference counterparts: cfg::configure_aligner (configuration/configure_aligner.hpp:165-206),
// cfg::method_global / method_local (method_global.hpp:121-145, method_local.hpp:118-137),
// cfg::gap_model_affine (gap_model_affine.hpp:130-155), cfg::score_model_unitary* rules
// (score_model_unitary.hpp:185-209, score_model_unitary_simd_saturated.hpp:259-284),
// end-gap policies (end_gap_policy.hpp:20-36), results (result/aligner_result_bulk.hpp:43-69).
// Every rule of the unitary family selects the same GB300 kernels; the width is
// chosen per pair on the device.  Errors throw std::runtime_error, as the
// reference's only runtime error does (tracker_global_simd_saturated.hpp:98-100).
#pragma once

#include <algorithm>
#include <array>
#include <concepts>
#include <cstddef>
#include <cstdint>
#include <memory>
#include <ranges>
#include <stdexcept>
#include <string>
#include <string_view>
#include <utility>
#include <vector>

#include "pairwise_aligner_gb300.h"

namespace seqan::pairwise_aligner_gb300 {
inline namespace v1 {

namespace cfg {

enum struct end_gap : bool { penalised, free };

struct leading_end_gap {
    end_gap first_column{end_gap::penalised};
    end_gap first_row{end_gap::penalised};
};

struct trailing_end_gap {
    end_gap last_column{end_gap::penalised};
    end_gap last_row{end_gap::penalised};
};

// Flattened configuration of a rule chain.
struct settings {
    bool has_method = false, has_gap = false, has_score = false;
    bool local = false;
    leading_end_gap leading{};
    trailing_end_gap trailing{};
    int32_t gap_open = 0, gap_extension = 0;
    int32_t match = 0, mismatch = 0;
    int32_t width_hint = 0;
    std::vector<uint8_t> matrix_symbols;     // score_model_matrix: symbol of each rank
    std::vector<int32_t> matrix_scores;      // ... and the flat dim x dim scores
};

struct initial_t {
    constexpr void apply(settings &) const noexcept {}
};
inline constexpr initial_t initial{};

template <typename pred_t, typename fn_t>
struct rule {
    pred_t predecessor;
    fn_t fn;
    constexpr void apply(settings &s) const
    {
        predecessor.apply(s);
        fn(s);
    }
};

template <typename pred_t, typename fn_t>
constexpr auto make_rule(pred_t pred, fn_t fn)
{
    return rule<pred_t, fn_t>{std::move(pred), std::move(fn)};
}

template <typename t>
concept configuration_rule = requires(t const &r, settings &s) { r.apply(s); };

inline constexpr struct method_global_fn {
    template <configuration_rule pred_t>
    constexpr auto operator()(pred_t pred, leading_end_gap lead = {}, trailing_end_gap trail = {}) const
    {
        return make_rule(std::move(pred), [lead, trail](settings &s) {
            if (s.has_method) throw std::runtime_error("configuration has more than one method rule");
            s.has_method = true;
            s.local = false;
            s.leading = lead;
            s.trailing = trail;
        });
    }
    constexpr auto operator()(leading_end_gap lead = {}, trailing_end_gap trail = {}) const
    {
        return (*this)(initial, lead, trail);
    }
} method_global{};

inline constexpr struct method_local_fn {
    template <configuration_rule pred_t>
    constexpr auto operator()(pred_t pred) const
    {
        return make_rule(std::move(pred), [](settings &s) {
            if (s.has_method) throw std::runtime_error("configuration has more than one method rule");
            s.has_method = true;
            s.local = true;                              // method_local.hpp:41-49: all end gaps free
            s.leading = {end_gap::free, end_gap::free};
            s.trailing = {end_gap::free, end_gap::free};
        });
    }
    constexpr auto operator()() const { return (*this)(initial); }
} method_local{};

inline constexpr struct gap_model_affine_fn {
    template <configuration_rule pred_t>
    constexpr auto operator()(pred_t pred, int32_t open, int32_t extension) const
    {
        return make_rule(std::move(pred), [open, extension](settings &s) {
            if (s.has_gap) throw std::runtime_error("configuration has more than one gap model");
            s.has_gap = true;
            s.gap_open = open;
            s.gap_extension = extension;
        });
    }
    constexpr auto operator()(int32_t open, int32_t extension) const { return (*this)(initial, open, extension); }
} gap_model_affine{};

struct score_model_unitary_fn {
    template <configuration_rule pred_t, std::integral score_t>
    constexpr auto operator()(pred_t pred, score_t match, score_t mismatch) const
    {
        const auto ma = static_cast<int32_t>(match), mi = static_cast<int32_t>(mismatch);
        return make_rule(std::move(pred), [ma, mi](settings &s) {
            if (s.has_score) throw std::runtime_error("configuration has more than one score model");
            s.has_score = true;
            s.match = ma;
            s.mismatch = mi;
        });
    }
    template <std::integral score_t>
    constexpr auto operator()(score_t match, score_t mismatch) const
    {
        return (*this)(initial, match, mismatch);
    }
};
inline constexpr score_model_unitary_fn score_model_unitary_gpu{};
inline constexpr score_model_unitary_fn score_model_unitary{};
inline constexpr score_model_unitary_fn score_model_unitary_simd{};
inline constexpr score_model_unitary_fn score_model_unitary_simd_saturated{};

// cfg::score_model_matrix(pred, matrix) (configuration/score_model_matrix.hpp:203-222): the
// same argument type as the reference, an array of (symbol, row of scores) pairs; the score
// of sequence1 symbol a against sequence2 symbol b is row(a)[rank(b)].
inline constexpr struct score_model_matrix_fn {
    template <configuration_rule pred_t, typename alphabet_t, std::integral score_t, size_t dim>
    auto operator()(pred_t pred, std::array<std::pair<alphabet_t, std::array<score_t, dim>>, dim> const &m) const
    {
        static_assert(dim >= 1 && dim <= 32, "the GB300 kernels take up to 32 symbols");
        std::array<uint8_t, dim> sym{};
        std::array<int32_t, dim * dim> sc{};
        for (size_t r = 0; r < dim; ++r) {
            sym[r] = static_cast<uint8_t>(m[r].first);
            for (size_t k = 0; k < dim; ++k) sc[r * dim + k] = static_cast<int32_t>(m[r].second[k]);
        }
        return make_rule(std::move(pred), [sym, sc](settings &s) {
            if (s.has_score) throw std::runtime_error("configuration has more than one score model");
            s.has_score = true;
            s.matrix_symbols.assign(sym.begin(), sym.end());
            s.matrix_scores.assign(sc.begin(), sc.end());
        });
    }
    template <typename alphabet_t, std::integral score_t, size_t dim>
    auto operator()(std::array<std::pair<alphabet_t, std::array<score_t, dim>>, dim> const &m) const
    {
        return (*this)(initial, m);
    }
} score_model_matrix{};

}  // namespace cfg

// One result: score(), the two sequences, and the 1-based end position.
class aligner_result {
public:
    aligner_result(std::shared_ptr<const std::string> s1, std::shared_ptr<const std::string> s2, uint64_t b1,
                   uint64_t l1, uint64_t b2, uint64_t l2, pa_result r)
        : _s1{std::move(s1)}, _s2{std::move(s2)}, _b1{b1}, _l1{l1}, _b2{b2}, _l2{l2}, _r{r}
    {}
    int32_t score() const noexcept { return _r.score; }
    std::string_view sequence1() const noexcept { return std::string_view{*_s1}.substr(_b1, _l1); }
    std::string_view sequence2() const noexcept { return std::string_view{*_s2}.substr(_b2, _l2); }
    std::pair<int32_t, int32_t> end_position() const noexcept { return {_r.end1, _r.end2}; }
    uint8_t width() const noexcept { return _r.width; }

private:
    std::shared_ptr<const std::string> _s1, _s2;
    uint64_t _b1, _l1, _b2, _l2;
    pa_result _r;
};

// A result with its alignment (aligner::compute_alignments): the 0-based cell the path starts
// after and one op per alignment column ('=', 'X', 'D': a sequence1 symbol against a gap,
// 'I': a sequence2 symbol against a gap).
class alignment_result : public aligner_result {
public:
    alignment_result(aligner_result base, pa_alignment a, std::string ops)
        : aligner_result{std::move(base)}, _a{a}, _ops{std::move(ops)}
    {}
    std::pair<int32_t, int32_t> begin_position() const noexcept { return {_a.begin1, _a.begin2}; }
    std::string_view ops() const noexcept { return _ops; }
    std::string cigar() const
    {
        std::string out;
        for (size_t k = 0; k < _ops.size();) {
            size_t e = k;
            while (e < _ops.size() && _ops[e] == _ops[k]) ++e;
            out += std::to_string(e - k);
            out += _ops[k];
            k = e;
        }
        return out;
    }

private:
    pa_alignment _a;
    std::string _ops;
};

class aligner {
public:
    explicit aligner(cfg::settings const &s, int device = 0)
    {
        if (!s.has_score) throw std::runtime_error("configuration lacks a score model (configure_aligner.hpp:176)");
        if (!s.has_gap) throw std::runtime_error("configuration lacks a gap model (configure_aligner.hpp:177)");
        _cfg.method = s.local ? PA_METHOD_LOCAL : PA_METHOD_GLOBAL;
        _cfg.match = s.match;
        _cfg.mismatch = s.mismatch;
        _cfg.gap_open = s.gap_open;
        _cfg.gap_extension = s.gap_extension;
        _cfg.first_column_free = s.leading.first_column == cfg::end_gap::free;
        _cfg.first_row_free = s.leading.first_row == cfg::end_gap::free;
        _cfg.last_column_free = s.trailing.last_column == cfg::end_gap::free;
        _cfg.last_row_free = s.trailing.last_row == cfg::end_gap::free;
        _cfg.width_hint = s.width_hint;
        _cfg.band_mode = 0;
        pa_ctx *c = nullptr;
        check(pa_create(&c, device, nullptr), nullptr);
        _ctx = std::shared_ptr<pa_ctx>(c, [](pa_ctx *p) { pa_destroy(p); });
        if (!s.matrix_symbols.empty()) {
            _cfg.method |= PA_SCORE_MATRIX;
            check(pa_set_substitution_matrix(_ctx.get(), s.matrix_symbols.data(),
                                             static_cast<uint32_t>(s.matrix_symbols.size()), s.matrix_scores.data()),
                  _ctx.get());
        }
    }

    // Bulk: ranges of character sequences, same length; any number of pairs.
    template <std::ranges::forward_range seqs1_t, std::ranges::forward_range seqs2_t>
        requires std::ranges::forward_range<std::ranges::range_reference_t<seqs1_t>>
    std::vector<aligner_result> compute(seqs1_t &&seqs1, seqs2_t &&seqs2)
    {
        auto [s1, o1] = pack(seqs1);
        auto [s2, o2] = pack(seqs2);
        if (o1.size() != o2.size()) throw std::runtime_error("both collections must hold the same number of sequences");
        const uint64_t n = o1.size() - 1;
        std::vector<pa_result> out(n);
        check(pa_align_batch(_ctx.get(), &_cfg, reinterpret_cast<const uint8_t *>(s1->data()), o1.data(),
                             reinterpret_cast<const uint8_t *>(s2->data()), o2.data(), n, out.data(), nullptr),
              _ctx.get());
        std::vector<aligner_result> res;
        res.reserve(n);
        for (uint64_t k = 0; k < n; ++k)
            res.emplace_back(s1, s2, o1[k], o1[k + 1] - o1[k], o2[k], o2[k + 1] - o2[k], out[k]);
        return res;
    }

    // Bulk with alignments (pa_traceback_batch): the same results plus begin cell and ops.
    template <std::ranges::forward_range seqs1_t, std::ranges::forward_range seqs2_t>
        requires std::ranges::forward_range<std::ranges::range_reference_t<seqs1_t>>
    std::vector<alignment_result> compute_alignments(seqs1_t &&seqs1, seqs2_t &&seqs2)
    {
        auto [s1, o1] = pack(seqs1);
        auto [s2, o2] = pack(seqs2);
        if (o1.size() != o2.size()) throw std::runtime_error("both collections must hold the same number of sequences");
        const uint64_t n = o1.size() - 1;
        std::vector<pa_result> out(n);
        std::vector<pa_alignment> aln(n);
        std::string ops(std::max<uint64_t>(o1.back() + o2.back(), 1), '\0');
        check(pa_traceback_batch(_ctx.get(), &_cfg, reinterpret_cast<const uint8_t *>(s1->data()), o1.data(),
                                 reinterpret_cast<const uint8_t *>(s2->data()), o2.data(), n, out.data(), aln.data(),
                                 reinterpret_cast<uint8_t *>(ops.data()), nullptr),
              _ctx.get());
        std::vector<alignment_result> res;
        res.reserve(n);
        for (uint64_t k = 0; k < n; ++k)
            res.emplace_back(aligner_result{s1, s2, o1[k], o1[k + 1] - o1[k], o2[k], o2[k + 1] - o2[k], out[k]}, aln[k],
                             ops.substr(o1[k] + o2[k], aln[k].n_ops));
        return res;
    }

    // Bulk over 2-bit packed DNA (pa_align_batch_packed; see pack_2bit): pair k is bases
    // [off1[k], off1[k+1]) of words1 against [off2[k], off2[k+1]) of words2.
    std::vector<pa_result> compute_packed(std::vector<uint32_t> const &words1, std::vector<uint64_t> const &off1,
                                          std::vector<uint32_t> const &words2, std::vector<uint64_t> const &off2)
    {
        if (off1.size() != off2.size() || off1.empty())
            throw std::runtime_error("both collections must hold the same number of sequences");
        if (words1.size() * 16 < off1.back() || words2.size() * 16 < off2.back())
            throw std::runtime_error("the packed words end before the last offset");
        const uint64_t n = off1.size() - 1;
        std::vector<pa_result> out(n);
        check(pa_align_batch_packed(_ctx.get(), &_cfg, words1.data(), off1.data(), words2.data(), off2.data(), n,
                                    out.data(), nullptr),
              _ctx.get());
        return out;
    }

    // Single pair (interface_one_to_one_single.hpp:44-67).
    aligner_result compute(std::string_view seq1, std::string_view seq2)
    {
        std::vector<std::string_view> a{seq1}, b{seq2};
        return compute(a, b).front();
    }

private:
    static void check(pa_status s, pa_ctx *c)
    {
        if (s != PA_OK) {
            std::string msg = pa_status_string(s);
            if (c && *pa_last_error(c)) msg += std::string(": ") + pa_last_error(c);
            throw std::runtime_error(msg);
        }
    }

    template <typename seqs_t>
    static std::pair<std::shared_ptr<std::string>, std::vector<uint64_t>> pack(seqs_t &&seqs)
    {
        auto data = std::make_shared<std::string>();
        std::vector<uint64_t> off{0};
        for (auto &&s : seqs) {
            for (auto &&c : s) data->push_back(static_cast<char>(c));
            off.push_back(data->size());
        }
        return {data, std::move(off)};
    }

    pa_config _cfg{};
    std::shared_ptr<pa_ctx> _ctx;
};

// ---- input path -------------------------------------------------------------------------------

// A FASTA / FASTQ file in the batch layout (pa_seqfile_*): record k is
// sequences.substr(offsets[k], offsets[k + 1] - offsets[k]); qualities likewise (FASTQ only).
struct sequence_file {
    std::vector<std::string> names;
    std::string sequences;
    std::vector<uint64_t> offsets{0};
    std::string qualities;

    size_t size() const noexcept { return names.size(); }
    std::string_view sequence(size_t k) const
    {
        return std::string_view{sequences}.substr(offsets[k], offsets[k + 1] - offsets[k]);
    }
};

namespace detail {
inline sequence_file take_seqfile(pa_seqfile *f)
{
    sequence_file out;
    const uint64_t n = pa_seqfile_count(f);
    const uint64_t *off = pa_seqfile_offsets(f);
    out.offsets.assign(off, off + n + 1);
    const uint8_t *seq = pa_seqfile_sequences(f);
    out.sequences.assign(reinterpret_cast<const char *>(seq), off[n]);
    if (const uint8_t *q = pa_seqfile_qualities(f)) out.qualities.assign(reinterpret_cast<const char *>(q), off[n]);
    out.names.reserve(n);
    for (uint64_t k = 0; k < n; ++k) out.names.emplace_back(pa_seqfile_name(f, k));
    pa_seqfile_free(f);
    return out;
}
}  // namespace detail

// Read a FASTA or FASTQ file; a malformed record throws with its line number.
inline sequence_file read_sequences(std::string const &path)
{
    pa_seqfile *f = nullptr;
    char err[256] = {};
    if (pa_seqfile_read(path.c_str(), &f, err, sizeof(err)) != PA_OK) throw std::runtime_error(err);
    return detail::take_seqfile(f);
}

inline sequence_file parse_sequences(std::string_view text)
{
    pa_seqfile *f = nullptr;
    char err[256] = {};
    if (pa_seqfile_parse(text.data(), text.size(), &f, err, sizeof(err)) != PA_OK) throw std::runtime_error(err);
    return detail::take_seqfile(f);
}

// 2-bit DNA words (16 bases per word, A/a 0, C/c 1, G/g 2, T/t 3); `invalid` counts other bytes.
inline std::vector<uint32_t> pack_2bit(std::string_view bases, uint64_t *invalid = nullptr)
{
    std::vector<uint32_t> words((bases.size() + 15) / 16);
    uint64_t bad = 0;
    pa_pack_2bit_host(reinterpret_cast<const uint8_t *>(bases.data()), bases.size(), words.data(), &bad);
    if (invalid) *invalid = bad;
    return words;
}

namespace cfg {
// cfg::configure_aligner(rule) -> aligner (configure_aligner.hpp:165-206).
template <configuration_rule rule_t>
aligner configure_aligner(rule_t const &r, int device = 0)
{
    settings s;
    r.apply(s);
    return aligner{s, device};
}
}  // namespace cfg

}  // inline namespace v1
}  // namespace seqan::pairwise_aligner_gb300
