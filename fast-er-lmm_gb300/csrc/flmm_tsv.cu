// Output tables of a scan as text, laid out the way the reference CLI writes them (fasterlmm/cli.py:100-161): the
// per-phenotype gwas.tsv (the 14 FaST-LMM single_snp columns, rows in ascending p order) and the one-column
// perms.tsv.  Host code: the result columns arrive in host memory after the device post-scan step; the caller runs
// one phenotype per thread (every entry point here is re-entrant and holds no lock).
//
// Numbers are written as Apache Arrow's CSV writer writes them (the reference writes through pyarrow.csv): the
// shortest decimal digit string that reads back to the same double, in fixed notation when the decimal exponent e
// of the leading digit satisfies -6 <= e < 10 and as d.ddde+X / d.ddde-X otherwise; NaN as "nan", infinities as
// "inf" / "-inf", zeros as "0" / "-0", nulls as empty fields, booleans as true / false.  The shortest digits come
// from std::to_chars (C++17, shortest round trip); only the notation is decided here.
#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "flmm_common.cuh"

namespace {

constexpr int kNumChars = 40;  // longest formatted double: "-" + 17 digits + "." + "e-308" and fixed forms < 40

// Shortest round-trip text of v in Arrow's notation; returns the length written to out (>= kNumChars bytes).
int format_double(double v, char* out) {
    if (std::isnan(v)) {
        std::memcpy(out, "nan", 3);
        return 3;
    }
    if (std::isinf(v)) {
        if (v < 0) {
            std::memcpy(out, "-inf", 4);
            return 4;
        }
        std::memcpy(out, "inf", 3);
        return 3;
    }
    if (v == 0.0) {
        if (std::signbit(v)) {
            std::memcpy(out, "-0", 2);
            return 2;
        }
        out[0] = '0';
        return 1;
    }
    char sci[48];
    const auto res = std::to_chars(sci, sci + sizeof(sci), v, std::chars_format::scientific);
    const char* end = res.ptr;
    // sci = [-]d[.ddd]e(+|-)XX
    const char* p = sci;
    int n = 0;
    if (*p == '-') {
        out[n++] = '-';
        ++p;
    }
    char digits[24];
    int nd = 0;
    while (p < end && *p != 'e') {
        if (*p != '.') digits[nd++] = *p;
        ++p;
    }
    int e = 0;
    bool eneg = false;
    if (p < end && *p == 'e') {
        ++p;
        if (*p == '-' || *p == '+') eneg = (*p++ == '-');
        while (p < end) e = e * 10 + (*p++ - '0');
    }
    if (eneg) e = -e;
    if (e >= -6 && e < 10) {
        if (e < 0) {
            out[n++] = '0';
            out[n++] = '.';
            for (int i = 0; i < -e - 1; ++i) out[n++] = '0';
            for (int i = 0; i < nd; ++i) out[n++] = digits[i];
        } else {
            for (int i = 0; i <= e; ++i) out[n++] = i < nd ? digits[i] : '0';
            if (nd > e + 1) {
                out[n++] = '.';
                for (int i = e + 1; i < nd; ++i) out[n++] = digits[i];
            }
        }
        return n;
    }
    out[n++] = digits[0];
    if (nd > 1) {
        out[n++] = '.';
        for (int i = 1; i < nd; ++i) out[n++] = digits[i];
    }
    out[n++] = 'e';
    out[n++] = e < 0 ? '-' : '+';
    const int ae = e < 0 ? -e : e;
    char eb[8];
    const auto er = std::to_chars(eb, eb + sizeof(eb), ae);
    for (const char* q = eb; q < er.ptr; ++q) out[n++] = *q;
    return n;
}

int format_int(int64_t v, char* out) {
    const auto r = std::to_chars(out, out + 24, v);
    return static_cast<int>(r.ptr - out);
}

// Buffered file writer: appends to a 4 MB buffer and writes it out when full.
class Out {
public:
    explicit Out(const char* path) : f_(std::fopen(path, "wb")) { buf_.reserve(kCap); }
    ~Out() {
        if (f_) std::fclose(f_);
    }
    bool ok() const { return f_ != nullptr && !err_; }
    char* reserve(size_t n) {
        if (buf_.size() + n > kCap) flush();
        const size_t at = buf_.size();
        buf_.resize(at + n);
        return buf_.data() + at;
    }
    void commit(char* start, size_t reserved, size_t used) {
        (void)start;
        buf_.resize(buf_.size() - (reserved - used));
    }
    void put(const char* s, size_t n) {
        char* d = reserve(n);
        std::memcpy(d, s, n);
    }
    void put(char c) { *reserve(1) = c; }
    void put_double(double v) {
        char* d = reserve(kNumChars);
        commit(d, kNumChars, static_cast<size_t>(format_double(v, d)));
    }
    void put_int(int64_t v) {
        char* d = reserve(24);
        commit(d, 24, static_cast<size_t>(format_int(v, d)));
    }
    void flush() {
        if (f_ && !buf_.empty() && std::fwrite(buf_.data(), 1, buf_.size(), f_) != buf_.size()) err_ = true;
        buf_.clear();
    }
    bool close() {
        flush();
        if (f_ && std::fclose(f_) != 0) err_ = true;
        f_ = nullptr;
        return !err_;
    }

private:
    static constexpr size_t kCap = size_t(4) << 20;
    std::FILE* f_;
    std::vector<char> buf_;
    bool err_ = false;
};

}  // namespace

extern "C" int flmm_format_f64(const double* v, int64_t n, char* buf, int64_t buf_bytes, int64_t* offsets) {
    FLMM_REQUIRE((v && buf && offsets) || n == 0, "flmm_format_f64: NULL argument");
    int64_t at = 0;
    if (offsets) offsets[0] = 0;
    char tmp[kNumChars];
    for (int64_t i = 0; i < n; ++i) {
        const int len = format_double(v[i], tmp);
        if (at + len > buf_bytes) return flmm::fail(FLMM_ERR_ARG, "flmm_format_f64: buffer of %lld bytes is too small",
                                                    static_cast<long long>(buf_bytes));
        std::memcpy(buf + at, tmp, len);
        at += len;
        offsets[i + 1] = at;
    }
    return FLMM_OK;
}

extern "C" int flmm_write_gwas_tsv(const char* path, int64_t M, const char* snp_ids, const int64_t* snp_offsets,
                                   const double* chrom, const double* pos, const double* g_var, double p_var,
                                   const double* pvalue, const double* beta, const double* se, const double* sfve,
                                   const double* nullh2, int64_t ld, const int64_t* order, int64_t ld_order,
                                   const char* pheno_name, int64_t pheno_count) {
    FLMM_REQUIRE(path && pheno_name && M >= 0, "flmm_write_gwas_tsv: bad arguments");
    FLMM_REQUIRE(M == 0 || (snp_ids && snp_offsets && chrom && pos && g_var && pvalue && beta && se && sfve &&
                                 nullh2 && ld >= 1 && (!order || ld_order >= 1)),
                 "flmm_write_gwas_tsv: NULL column or bad stride");
    Out out(path);
    if (!out.ok()) return flmm::fail(FLMM_ERR_IO, "flmm_write_gwas_tsv: cannot open %s", path);
    static const char kHeader[] =
        "sid_index\tSNP\tChr\tGenDist\tChrPos\tPValue\tSnpWeight\tSnpWeightSE\tEffectSize\tSnpFractVarExpl\tMixing\t"
        "Nullh2\tPheno\tPhenoCount\n";
    out.put(kHeader, sizeof(kHeader) - 1);
    const size_t name_len = std::strlen(pheno_name);
    for (int64_t i = 0; i < M; ++i) {
        const int64_t v = order ? order[i * ld_order] : i;
        if (v < 0 || v >= M) return flmm::fail(FLMM_ERR_ARG, "flmm_write_gwas_tsv: order holds %lld, outside [0, %lld)",
                                               static_cast<long long>(v), static_cast<long long>(M));
        const int64_t o = v * ld;
        const double b = beta[o];
        const double effect = b * b * g_var[v] / p_var;  // EffectSize, evaluated left to right as numpy does
        out.put_int(v);
        out.put('\t');
        out.put(snp_ids + snp_offsets[v], static_cast<size_t>(snp_offsets[v + 1] - snp_offsets[v]));
        out.put('\t');
        out.put_double(chrom[v]);
        out.put("\t\t", 2);  // GenDist is null
        out.put_double(pos[v]);
        out.put('\t');
        out.put_double(pvalue[o]);
        out.put('\t');
        out.put_double(b);
        out.put('\t');
        out.put_double(se[o]);
        out.put('\t');
        out.put_double(effect);
        out.put('\t');
        out.put_double(sfve[o]);
        out.put("\t0\t", 3);  // Mixing
        out.put_double(nullh2[o]);
        out.put('\t');
        out.put(pheno_name, name_len);
        out.put('\t');
        out.put_int(pheno_count);
        out.put('\n');
    }
    if (!out.close()) return flmm::fail(FLMM_ERR_IO, "flmm_write_gwas_tsv: write to %s failed", path);
    return FLMM_OK;
}

extern "C" int flmm_write_column_tsv(const char* path, const char* header, const double* v, int64_t n) {
    FLMM_REQUIRE(path && header && (v || n == 0) && n >= 0, "flmm_write_column_tsv: bad arguments");
    Out out(path);
    if (!out.ok()) return flmm::fail(FLMM_ERR_IO, "flmm_write_column_tsv: cannot open %s", path);
    out.put(header, std::strlen(header));
    out.put('\n');
    for (int64_t i = 0; i < n; ++i) {
        out.put_double(v[i]);
        out.put('\n');
    }
    if (!out.close()) return flmm::fail(FLMM_ERR_IO, "flmm_write_column_tsv: write to %s failed", path);
    return FLMM_OK;
}
