// Zheng07 HOD mocks drawn on the GPU: many realisations of one halo table, one
// per parameter vector theta = (logMmin, sigma_logM, logM0, logM1, alpha), as
// halotools' mock population does for the Zheng07 model
// (empirical_models/factories/hod_mock_factory.py:196-401 with
// zheng07_components.py:149-153, 455-470 and the NFW satellite profile), without
// a host round trip: the galaxies land in one device buffer, mock m in rows
// [offsets[m], offsets[m+1]), ready for the batched pair counter.
//
// Pass 1 (k_hod_count), one thread per (theta, halo): a Bernoulli central with
// probability <Ncen> = (1 + erf((log10 M - logMmin) / sigma_logM)) / 2 and a
// Poisson number of satellites with mean <Nsat> = ((M - M0) / M1)^alpha for
// M > M0.  An exclusive scan of the counts gives every (theta, halo) its rows.
// Pass 2 (k_hod_write) repeats the same draws, writes the central at the halo
// centre and each satellite at an NFW radius (the enclosed-mass profile
// ln(1+x) - x/(1+x) inverted by bisection, x = r c / R_vir) in an isotropic
// direction, wrapped into the periodic box.
//
// Random numbers: Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random
// numbers: as easy as 1, 2, 3", SC 2011), keyed by the seed and counted by
// (halo, theta, draw, stream): every draw is fixed by its indices, whatever the
// launch shape.  Poisson variates: sequential inversion for means below 10, else
// the transformed rejection of Hormann ("The transformed rejection method for
// generating Poisson random variables", Insurance: Mathematics and Economics 12,
// 1993), as numpy's sampler does.
#include "gbp_device.cuh"

struct HodTheta {
    double logMmin, inv_sigma, M0, inv_M1, alpha;
};

struct P4 {
    unsigned x, y, z, w;
};

__device__ __forceinline__ P4 philox4x32_10(P4 c, unsigned k0, unsigned k1) {
#pragma unroll
    for (int r = 0; r < 10; r++) {
        const unsigned lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
        const unsigned lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
        c = P4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return c;
}

// (0, 1) with 53 random bits from two words
__device__ __forceinline__ double u01(unsigned a, unsigned b) {
    return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6) + 0.5) * 0x1p-53;
}

// Uniform stream of one (theta, halo): two doubles per Philox block
struct HodRng {
    unsigned k0, k1, halo, theta, n;
    double buf[2];
    int have;
    __device__ double next() {
        if (have == 0) {
            const P4 r = philox4x32_10(P4{halo, theta, n++, 0u}, k0, k1);
            buf[0] = u01(r.x, r.y);
            buf[1] = u01(r.z, r.w);
            have = 2;
        }
        return buf[--have];
    }
};

__device__ int poisson(HodRng &g, double mu) {
    if (!(mu > 0.0)) return 0;
    if (mu < 10.0) {
        // inversion: the smallest k with F(k) >= u
        const double u = g.next();
        double p = exp(-mu), F = p;
        int k = 0;
        while (u > F && k < 1000) {
            k++;
            p *= mu / k;
            F += p;
        }
        return k;
    }
    // transformed rejection (PTRS)
    const double smu = sqrt(mu), b = 0.931 + 2.53 * smu, a = -0.059 + 0.02483 * b;
    const double inv_alpha = 1.1239 + 1.1328 / (b - 3.4), vr = 0.9277 - 3.6224 / (b - 2.0);
    const double lmu = log(mu);
    for (int it = 0; it < 1000; it++) {
        const double U = g.next() - 0.5, V = g.next();
        const double us = 0.5 - fabs(U);
        const double k = floor((2.0 * a / us + b) * U + mu + 0.43);
        if (us >= 0.07 && V <= vr) return (int)k;
        if (k < 0.0 || (us < 0.013 && V > us)) continue;
        if (log(V) + log(inv_alpha) - log(a / (us * us) + b) <= -mu + k * lmu - lgamma(k + 1.0))
            return (int)k;
    }
    return (int)floor(mu + 0.5);  // (never reached in practice: the acceptance rate is ~0.9)
}

// central (0/1) and satellite count of halo i under theta t, from the stream
// (the mean occupations in FP32: ample for drawing, and GB300's FP64 units are slow)
__device__ __forceinline__ int2 hod_draw(HodRng &g, const HodTheta &t, double logm, double mass) {
    const float ncen = 0.5f * (1.0f + erff((float)((logm - t.logMmin) * t.inv_sigma)));
    const int cen = g.next() < (double)ncen ? 1 : 0;
    const float nsat = mass > t.M0 ? powf((float)((mass - t.M0) * t.inv_M1), (float)t.alpha) : 0.0f;
    return make_int2(cen, poisson(g, (double)nsat));
}

__global__ void k_hod_logm(const double *mass, int64_t n, double *logm) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        logm[i] = log10(mass[i]);
}

__global__ void k_hod_count(const double *mass, const double *logm, int64_t nh,
                            const HodTheta *th, int nth, unsigned k0, unsigned k1, int *count) {
    const int64_t total = nh * nth;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int m = (int)(t / nh);
        const int64_t i = t - (int64_t)m * nh;
        HodRng g{k0, k1, (unsigned)i, (unsigned)m, 0u, {0.0, 0.0}, 0};
        const int2 d = hod_draw(g, th[m], logm[i], mass[i]);
        count[t] = d.x + d.y;
    }
}

// x with ln(1+x) - x/(1+x) = u (ln(1+c) - c/(1+c)), 0 < x < c
__device__ __forceinline__ float nfw_x(float u, float c) {
    const float target = u * (log1pf(c) - c / (1.0f + c));
    float lo = 0.0f, hi = c;
#pragma unroll 1
    for (int it = 0; it < 40; it++) {
        const float mid = 0.5f * (lo + hi);
        if (log1pf(mid) - mid / (1.0f + mid) < target) lo = mid;
        else hi = mid;
    }
    return 0.5f * (lo + hi);
}

// into [0, L); an FP32 value that rounds up to L is its periodic image 0
__device__ __forceinline__ float wrap(double v, double L) {
    double r = fmod(v, L);
    if (r < 0.0) r += L;
    if (r >= L) r -= L;
    const float f = (float)r;
    return f >= (float)L ? 0.0f : f;
}

__global__ void k_hod_write(const double *xyz, const double *mass, const double *logm,
                            const double *conc, const double *rvir, int64_t nh,
                            const HodTheta *th, int nth, unsigned k0, unsigned k1,
                            const int *off, double L, float *gal) {
    const int64_t total = nh * nth;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        int64_t o = off[t];
        const int64_t end = off[t + 1];
        if (o == end) continue;
        const int m = (int)(t / nh);
        const int64_t i = t - (int64_t)m * nh;
        HodRng g{k0, k1, (unsigned)i, (unsigned)m, 0u, {0.0, 0.0}, 0};
        const int2 d = hod_draw(g, th[m], logm[i], mass[i]);
        const double cx = xyz[3 * i], cy = xyz[3 * i + 1], cz = xyz[3 * i + 2];
        if (d.x && o < end) {
            gal[3 * o] = wrap(cx, L);
            gal[3 * o + 1] = wrap(cy, L);
            gal[3 * o + 2] = wrap(cz, L);
            o++;
        }
        const float c = (float)conc[i], rv = (float)rvir[i];
        for (unsigned s = 0; o < end; s++, o++) {
            // satellite s: its own Philox block (stream 1)
            const P4 r = philox4x32_10(P4{(unsigned)i, (unsigned)m, s, 1u}, k0, k1);
            const float ur = (float)u01(r.x, r.y);
            const float mu = 2.0f * ((float)(r.z >> 8) * 0x1p-24f) - 1.0f;
            const float ph = 6.283185307179586f * ((float)(r.w >> 8) * 0x1p-24f);
            const float rad = nfw_x(ur, c) / c * rv;
            const float sn = sqrtf(fmaxf(0.0f, 1.0f - mu * mu));
            float sp, cp;
            sincosf(ph, &sp, &cp);
            gal[3 * o] = wrap(cx + (double)(rad * sn * cp), L);
            gal[3 * o + 1] = wrap(cy + (double)(rad * sn * sp), L);
            gal[3 * o + 2] = wrap(cz + (double)(rad * mu), L);
        }
    }
}

static unsigned grid_for(int64_t n) {
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 16));
}

cudaError_t gbp_hod_count(const double *mass, double *logm, int64_t nh, const void *thetas,
                          int nth, unsigned long long seed, int *count, cudaStream_t st) {
    k_hod_logm<<<grid_for(nh), 256, 0, st>>>(mass, nh, logm);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_hod_count<<<grid_for(nh * nth), 256, 0, st>>>(mass, logm, nh, (const HodTheta *)thetas, nth,
                                                    (unsigned)seed, (unsigned)(seed >> 32), count);
    return cudaGetLastError();
}

cudaError_t gbp_hod_write(const double *xyz, const double *mass, const double *logm,
                          const double *conc, const double *rvir, int64_t nh, const void *thetas,
                          int nth, unsigned long long seed, const int *off, double L, float *gal,
                          cudaStream_t st) {
    k_hod_write<<<grid_for(nh * nth), 256, 0, st>>>(xyz, mass, logm, conc, rvir, nh,
                                                    (const HodTheta *)thetas, nth, (unsigned)seed,
                                                    (unsigned)(seed >> 32), off, L, gal);
    return cudaGetLastError();
}

size_t gbp_hod_theta_bytes() { return sizeof(HodTheta); }

// host: theta rows -> the derived constants the kernels use
void gbp_hod_thetas(const double *theta, int nth, void *out) {
    HodTheta *t = (HodTheta *)out;
    for (int m = 0; m < nth; m++) {
        const double *p = theta + 5 * (size_t)m;
        t[m].logMmin = p[0];
        t[m].inv_sigma = 1.0 / p[1];
        t[m].M0 = std::pow(10.0, p[2]);
        t[m].inv_M1 = 1.0 / std::pow(10.0, p[3]);
        t[m].alpha = p[4];
    }
}
