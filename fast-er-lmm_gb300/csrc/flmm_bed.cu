// PLINK .bed genotype decode on the device (the reference reads .bed through pysnptools, fasterlmm/io.py:54-67 and
// fasterlmm/io_stream.py:60-71).
//
// A SNP-major .bed stores, after its 3-byte header, one record of ceil(n_fam / 4) bytes per variant, four samples
// per byte from the least significant bit pair up: 00 homozygous for the first (A1) allele, 01 missing, 10
// heterozygous, 11 homozygous for the second allele.  Counting A1 alleles (count_A1, the reference's default) maps
// 00, 10, 11 to 2, 1, 0; counting A2 maps them to 0, 1, 2; missing becomes -1, the int8 dosage layout that
// flmm_standardise_dosage standardises.
#include <stdint.h>

#include "flmm_common.cuh"

using namespace flmm;

namespace {

// G[v, i] for kept sample i (row rows[i] of the .fam order, or i itself when rows is NULL) of variant v; a row
// outside [0, n_fam) reads as missing instead of outside the record
__global__ void k_bed_decode(const uint8_t* __restrict__ bed, int64_t bytes_per_variant, int n_variants, int n_fam,
                             const int32_t* __restrict__ rows, int n_keep, int count_a1, int8_t* __restrict__ G,
                             int64_t ldg) {
    const int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (t >= static_cast<int64_t>(n_variants) * n_keep) return;
    const int64_t v = t / n_keep;
    const int i = static_cast<int>(t % n_keep);
    const int r = rows ? rows[i] : i;
    if (r < 0 || r >= n_fam) {
        G[v * ldg + i] = -1;
        return;
    }
    const unsigned code = (bed[v * bytes_per_variant + (r >> 2)] >> (2 * (r & 3))) & 3u;
    int8_t d;
    if (code == 1u) {
        d = -1;
    } else {
        const int a2 = code == 0u ? 0 : (code == 2u ? 1 : 2);  // copies of the second allele
        d = static_cast<int8_t>(count_a1 ? 2 - a2 : a2);
    }
    G[v * ldg + i] = d;
}

}  // namespace

extern "C" int flmm_bed_decode(const uint8_t* bed, int64_t bytes_per_variant, int n_variants, int n_fam,
                               const int32_t* rows, int n_keep, int count_a1, int8_t* G, int64_t ldg, void* stream) {
    FLMM_REQUIRE((bed && G && n_fam > 0 && bytes_per_variant == (n_fam + 3) / 4 && n_keep >= 0 && ldg >= n_keep) ||
                     n_variants == 0,
                 "flmm_bed_decode: bad arguments (bytes_per_variant must be ceil(n_fam / 4))");
    FLMM_REQUIRE(rows || n_keep <= n_fam, "flmm_bed_decode: more samples than the .fam holds");
    const int64_t n = static_cast<int64_t>(n_variants) * n_keep;
    if (n == 0) return FLMM_OK;
    k_bed_decode<<<ceil_div(n, 256), 256, 0, as_stream(stream)>>>(bed, bytes_per_variant, n_variants, n_fam, rows,
                                                                   n_keep, count_a1, G, ldg);
    return check_launch("k_bed_decode");
}
