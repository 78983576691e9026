// fpconv.cuh -- FP64 <-> FP32 conversions in integer arithmetic, rounding to
// nearest even exactly as the hardware conversions do.  On GB300 the FP64
// unit, which also executes the hardware conversions, is narrow; kernels that
// convert every sample (the tensor-core transforms read and write FP64
// arrays but compute in FP32) use these instead.  The fast forms cover the
// normal range and zero; anything else (FP32 subnormals, overflow, inf, nan)
// reports false and the caller converts in hardware.
//
// Host-compilable (g++) so the CPU tests can check them against the host's
// conversions.
#pragma once

#ifdef __CUDACC__
#define FPC_HD __host__ __device__ __forceinline__
#else
#define FPC_HD inline
#endif

namespace fpc {

typedef unsigned long long u64;
typedef unsigned int u32;

// FP32 bits of RN(x) for the FP64 bits b; false outside zero and the normal FP32 range
FPC_HD bool f64_to_f32_bits(u64 b, u32 &out)
{
    const u32 hi = (u32)(b >> 32);
    const u32 sign = hi & 0x80000000u;
    // FP32 biased exponent e - 896 must lie in [1, 254]: e in [897, 1150]
    if ((hi & 0x7FFFFFFFu) - (897u << 20) >= (254u << 20)) {
        if ((b << 1) == 0) {  // +-0
            out = sign;
            return true;
        }
        return false;
    }
    // round to nearest even at bit 29: add half a unit less one, plus the kept last bit; the
    // rounded significand's carry runs into the exponent field (up to inf past the largest float)
    const u64 a = (b & 0x7FFFFFFFFFFFFFFFull) + 0x0FFFFFFFull + ((b >> 29) & 1u);
    // bits 29.. of a are (e << 23) | fraction; rebias mod 2^32 (the result is below 2^31)
    out = ((u32)(a >> 29) - (896u << 23)) + sign;
    return true;
}

// FP64 bits of the FP32 value with bits u (exact); false for subnormals, inf and nan
FPC_HD bool f32_to_f64_bits(u32 u, u64 &out)
{
    if ((u << 1) - 0x01000000u >= 0xFE000000u) {  // biased exponent 0 or 255
        if ((u << 1) == 0) {
            out = (u64)(u & 0x80000000u) << 32;
            return true;
        }
        return false;
    }
    const u32 hi = (u & 0x80000000u) + ((u & 0x7FFFFFFFu) >> 3) + (896u << 20);
    out = ((u64)hi << 32) | (u64)(u << 29);
    return true;
}

}  // namespace fpc
