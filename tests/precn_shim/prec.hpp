// Test stand-in for preclib's prec.hpp: just the number type and the two
// multiplier declarations that prec_gpu_precn.cpp needs, so the interposer
// can be built and run where preclib's sources are absent.  The field order
// and the zero convention (one allocated limb, a[0] = 0, rsiz 0) follow
// preclib's precn_t (prec.hpp:49-84, init_basic.cpp:47-52, 133).
#pragma once
#include <cstddef>
#include <cstdint>

struct precn_t {
    size_t asiz;  // allocated limbs
    size_t rsiz;  // used limbs (no zero top limb)
    uint64_t* a;
    precn_t();
    precn_t(const precn_t&) = delete;
    precn_t(precn_t&& o);
    precn_t& operator=(const precn_t&) = delete;
    ~precn_t();
};

precn_t mul_ntt(const precn_t& a, const precn_t& b);
precn_t mul_fft(const precn_t& a, const precn_t& b);

#if defined(COUNT_FFTS) && COUNT_FFTS
extern uint64_t total_fftmuls;
extern uint64_t danger_fftmuls;
extern uint64_t danger_fftmuls_1_4;
extern uint64_t danger_fftmuls_3_8;
extern double max_fft_rounding_error;
#endif
