// Philox4x32-10 counter-based generator, written from Salmon, Moraes, Dror and Shaw,
// "Parallel Random Numbers: As Easy as 1, 2, 3" (SC'11), section 3 and table 2.
// One header for host (oracle, tests) and device (kernels, NVRTC source); it includes nothing.
//
// Stream layout used by the simulator (keyed per run, counted per trajectory):
//   key     = (seed_lo, seed_hi)
//   counter = (c0, c1, traj_lo, traj_hi)
//   step s of a trajectory: c0 = s_lo, c1 = s_hi            -> words: dt, pick_hi, pick_lo, unused
//   initial state block b:  c0 = b,    c1 = 0xFFFFFFFF      -> nodes 4b .. 4b+3
// The reference draws from curand XORWOW per batch slot (src/jit_kernels/simulation.cu:23-32);
// a counter-based stream keyed by trajectory id makes every trajectory re-runnable on its own.
#pragma once

#ifdef __CUDACC__
#define MBG_HD __host__ __device__ __forceinline__
#else
#define MBG_HD inline
#endif

namespace mbg {

struct u32x4 {
    unsigned int x, y, z, w;
};

MBG_HD void philox_mulhilo(unsigned int a, unsigned int b, unsigned int& hi, unsigned int& lo) {
#ifdef __CUDA_ARCH__
    lo = a * b;
    hi = __umulhi(a, b);
#else
    unsigned long long p = (unsigned long long)a * (unsigned long long)b;
    lo = (unsigned int)p;
    hi = (unsigned int)(p >> 32);
#endif
}

MBG_HD u32x4 philox4x32_10(u32x4 c, unsigned int k0, unsigned int k1) {
#ifdef __CUDA_ARCH__
#pragma unroll
#endif
    for (int r = 0; r < 10; ++r) {
        unsigned int hi0, lo0, hi1, lo1;
        philox_mulhilo(0xD2511F53u, c.x, hi0, lo0);
        philox_mulhilo(0xCD9E8D57u, c.z, hi1, lo1);
        u32x4 n;
        n.x = hi1 ^ c.y ^ k0;
        n.y = lo1;
        n.z = hi0 ^ c.w ^ k1;
        n.w = lo0;
        c = n;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return c;
}

// Draws of one Gillespie step of trajectory `traj`.
MBG_HD u32x4 philox_step(unsigned long long seed, unsigned long long traj, unsigned long long step) {
    u32x4 c = {(unsigned int)step, (unsigned int)(step >> 32), (unsigned int)traj, (unsigned int)(traj >> 32)};
    return philox4x32_10(c, (unsigned int)seed, (unsigned int)(seed >> 32));
}

// Draws for the initial state of nodes 4*block .. 4*block+3.
MBG_HD u32x4 philox_init(unsigned long long seed, unsigned long long traj, unsigned int block) {
    u32x4 c = {block, 0xFFFFFFFFu, (unsigned int)traj, (unsigned int)(traj >> 32)};
    return philox4x32_10(c, (unsigned int)seed, (unsigned int)(seed >> 32));
}

// Uniform in (0, 1] with 24 significant bits; exact in float and double.
MBG_HD float u01_open0_f(unsigned int u) { return (float)((u >> 8) + 1u) * (1.0f / 16777216.0f); }
MBG_HD double u01_open0_d(unsigned int u) { return (double)((u >> 8) + 1u) * (1.0 / 16777216.0); }

// Node pick: r = floor(U64 * total / 2^64) with U64 = (hi << 32) | lo, so r is uniform on
// [0, total) and node i is picked with probability rate_i / total, exactly.
MBG_HD unsigned long long pick_target(unsigned int hi, unsigned int lo, unsigned long long total) {
    unsigned long long u = ((unsigned long long)hi << 32) | lo;
#ifdef __CUDA_ARCH__
    return __umul64hi(u, total);
#else
    return (unsigned long long)(((unsigned __int128)u * total) >> 64);
#endif
}

}  // namespace mbg
