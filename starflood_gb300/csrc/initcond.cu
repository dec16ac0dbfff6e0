// initcond.cu -- initcond_generate (src/initcond.c:11-255) on the device: the
// reference's default initial conditions, one thread per body.
//
//   mass     (4/3) pi radius^2 / N for radius 1 (the reference's formula,
//            radius squared, kept as it is)
//   position uniform in the unit ball: direction from pcg4d({0xD88D5EFD+i,
//            0x203F83D3, 0x710BE493, 0xA294E7F1}), radius cbrt(u)
//   velocity a Gaussian speed (sigma 1e-4, Box-Muller on the hash of
//            {0x4AFDC7CF+i, 0xAE8D7CF2, 0xE4827F00, 0xE44CA389}) in a direction
//            from a second round of that hash, plus 4e-3 sqrt(8 pi G / 3) x
//   rad      0.1 (with SPH)
//
// FP64 as in the reference, every product and sum rounded separately (no
// contraction); cos / sin / acos / cbrt / log are CUDA's, within an ulp of
// the host libm's, so a coordinate can differ from the host build's in its
// last FP32 bit when the FP64 value lies within an ulp of a rounding edge.
#include "internal.cuh"

namespace {

constexpr double IC_TAU = 6.28318530717958647692528676655900576839433879875021;
constexpr double IC_PI_4_3 = 4.18879020478639098461685784437267051226289253250014;
constexpr double IC_PI_8_3 = 8.37758040957278196923371568874534102452578506500028;
constexpr double IC_INV_PCG = 2.3283062977608182109179324470460414886474609375e-10;  // INV_PCG32_MAX

__device__ __forceinline__ void unit_direction(uint32_t a, uint32_t b, double& x, double& y, double& z) {
    const double r0 = __dmul_rn(IC_INV_PCG, (double)a), r1 = __dmul_rn(IC_INV_PCG, (double)b);
    const double phi = __dmul_rn(IC_TAU, r0);
    const double the = acos(__dsub_rn(__dmul_rn(2.0, r1), 1.0));
    const double cp = cos(phi), sp = sin(phi), ct = cos(the), st = sin(the);
    x = __dmul_rn(cp, st);
    y = __dmul_rn(sp, st);
    z = ct;
}

__global__ void k_initcond(float* __restrict__ slab, uint32_t n, uint32_t dof, double G) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float* pos = slab;
    float* vel = slab + (size_t)3 * n;
    float* mas = slab + (size_t)9 * n;
    // initcond.c:27-44
    const double radius = 1.000;
    const double volume = __dmul_rn(IC_PI_4_3, __dmul_rn(radius, radius));
    mas[i] = (float)__ddiv_rn(volume, (double)n);
    if (dof >= 16) slab[(size_t)13 * n + i] = 0.100f;
    // initcond.c:47-118: position
    uint32_t s0 = 0xD88D5EFDu + i, s1 = 0x203F83D3u, s2 = 0x710BE493u, s3 = 0xA294E7F1u;
    pcg4d(s0, s1, s2, s3);
    double px, py, pz;
    unit_direction(s0, s1, px, py, pz);
    const double scale = __dmul_rn(radius, cbrt(__dmul_rn(IC_INV_PCG, (double)s2)));
    const float fx = (float)__dmul_rn(px, scale), fy = (float)__dmul_rn(py, scale), fz = (float)__dmul_rn(pz, scale);
    pos[3u * i] = fx;
    pos[3u * i + 1u] = fy;
    pos[3u * i + 2u] = fz;
    // initcond.c:121-215: velocity, from the stored FP32 position
    uint32_t t0 = 0x4AFDC7CFu + i, t1 = 0xAE8D7CF2u, t2 = 0xE4827F00u, t3 = 0xE44CA389u;
    pcg4d(t0, t1, t2, t3);
    const double u0 = __dmul_rn(IC_INV_PCG, (double)t0), u1 = __dmul_rn(IC_INV_PCG, (double)t1);
    const double u2 = __dmul_rn(IC_INV_PCG, (double)t2), u3 = __dmul_rn(IC_INV_PCG, (double)t3);
    const double a0 = sqrt(__dmul_rn(-2.0, log(u0))), a2 = sqrt(__dmul_rn(-2.0, log(u2)));
    const double sigma = 1.000e-4;
    const double n0 = __dmul_rn(__dmul_rn(a0, cos(__dmul_rn(IC_TAU, u1))), sigma);
    const double n1 = __dmul_rn(__dmul_rn(a0, sin(__dmul_rn(IC_TAU, u1))), sigma);
    const double n2 = __dmul_rn(__dmul_rn(a2, cos(__dmul_rn(IC_TAU, u3))), sigma);
    const double speed = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(n0, n0), __dmul_rn(n1, n1)), __dmul_rn(n2, n2)));
    pcg4d(t0, t1, t2, t3);
    double vx, vy, vz;
    unit_direction(t0, t1, vx, vy, vz);
    vx = __dmul_rn(vx, speed);
    vy = __dmul_rn(vy, speed);
    vz = __dmul_rn(vz, speed);
    const double h = __dmul_rn(4.000e-3, sqrt(__dmul_rn(IC_PI_8_3, G)));
    vel[3u * i] = (float)__dadd_rn(vx, __dmul_rn(h, (double)fx));
    vel[3u * i + 1u] = (float)__dadd_rn(vy, __dmul_rn(h, (double)fy));
    vel[3u * i + 2u] = (float)__dadd_rn(vz, __dmul_rn(h, (double)fz));
}

}  // namespace

extern "C" int sfgpu_initcond(sfgpu_sim* s) {
    sf_clear_error();
    if (!s) {
        sf_set_error("sfgpu_initcond: simulation is NULL");
        return SFGPU_FAILURE;
    }
    if (s->n == 0) return SFGPU_OK;
    k_initcond<<<sf_ceil_div(s->n, 256), 256, 0, s->stream>>>(s->slab, s->n, s->dof, s->p.G);
    SF_CHECK_LAUNCH();
    return sf_refresh_fp64(s);
}
