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
    const u32 hi = (u32)(b >> 32), lo = (u32)b;
    const u32 sign = hi & 0x80000000u;
    if ((b << 1) == 0) {  // +-0
        out = sign;
        return true;
    }
    const u32 e = (hi >> 20) & 0x7FFu;
    // FP32 biased exponent e - 896 must lie in [1, 254]
    if (e - 897u > 253u) return false;
    const u32 m = ((hi & 0xFFFFFu) << 3) | (lo >> 29);  // the top 23 fraction bits
    const u32 rem = lo & 0x1FFFFFFFu;                   // the 29 dropped bits
    u32 r = ((e - 896u) << 23) | m;
    r += (u32)((rem > 0x10000000u) | ((rem == 0x10000000u) & (m & 1u)));  // a carry bumps the exponent
    out = sign | r;
    return true;
}

// FP64 bits of the FP32 value with bits u (exact); false for subnormals, inf and nan
FPC_HD bool f32_to_f64_bits(u32 u, u64 &out)
{
    const u32 sign = u & 0x80000000u;
    if ((u << 1) == 0) {
        out = (u64)sign << 32;
        return true;
    }
    const u32 E = (u >> 23) & 0xFFu;
    if (E - 1u > 253u) return false;
    const u32 hi = sign | ((E + 896u) << 20) | ((u & 0x7FFFFFu) >> 3);
    out = ((u64)hi << 32) | (u64)(u << 29);
    return true;
}

}  // namespace fpc
