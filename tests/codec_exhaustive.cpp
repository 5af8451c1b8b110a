// Exhaustive check of the library's Float16C codec (compiled for the host from the CUDA header)
// against the oracle's restatement: every 16-bit code decoded, every 32-bit pattern encoded.
#include <cstdio>
#include <cstdint>
#include <vector>
#include "../mojo_lbm_gb300/csrc/lbm_device.cuh"
extern "C" void oracle_f16c_encode(const float* in, uint16_t* out, int64_t n);
extern "C" void oracle_f16c_decode(const uint16_t* in, float* out, int64_t n);
int main() {
    std::vector<uint16_t> codes(65536);
    for (int i = 0; i < 65536; ++i) codes[i] = (uint16_t)i;
    std::vector<float> ref(65536);
    oracle_f16c_decode(codes.data(), ref.data(), 65536);
    long bad = 0;
    for (int i = 0; i < 65536; ++i) bad += lbm::as_u32(lbm::f16c_decode(i)) != lbm::as_u32(ref[i]);
    const uint64_t CH = 1ull << 24;
    long ebad = 0;
    std::vector<float> in(CH);
    std::vector<uint16_t> out(CH);
    for (uint64_t base = 0; base < (1ull << 32); base += CH) {
        for (uint64_t i = 0; i < CH; ++i) in[i] = lbm::as_f32((uint32_t)(base + i));
        oracle_f16c_encode(in.data(), out.data(), CH);
        long lb = 0;
#pragma omp parallel for reduction(+ : lb)
        for (int64_t i = 0; i < (int64_t)CH; ++i) lb += (uint16_t)lbm::f16c_encode(in[i]) != out[i];
        ebad += lb;
    }
    printf("decode mismatches %ld, encode mismatches %ld\n", bad, ebad);
    return (bad || ebad) ? 1 : 0;
}
