/*
 * Host-side random sequential addition (RSA) of spheres in a periodic box, used
 * to generate seeded synthetic configurations.  Sphere i (radius r[i], taken in
 * the given order) is placed at the first uniformly drawn position that does
 * not overlap any earlier sphere (contact at r_i + r_j).  Overlap checks go
 * through a cell grid whose edge is at least the largest contact distance.
 * Random numbers: xoshiro256** seeded through splitmix64.
 *
 * Returns 0 on success, 1 if a sphere found no place within max_tries draws,
 * 2 on allocation failure, 3 on a cell-capacity overflow.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>

static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

typedef struct {
    uint64_t s[4];
} rng_t;

static uint64_t splitmix(uint64_t *z) {
    uint64_t r = (*z += 0x9e3779b97f4a7c15ULL);
    r = (r ^ (r >> 30)) * 0xbf58476d1ce4e5b9ULL;
    r = (r ^ (r >> 27)) * 0x94d049bb133111ebULL;
    return r ^ (r >> 31);
}

static uint64_t next(rng_t *g) {
    uint64_t *s = g->s;
    const uint64_t result = rotl(s[1] * 5, 7) * 9;
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return result;
}

static double uniform(rng_t *g) { return (double)(next(g) >> 11) * (1.0 / 9007199254740992.0); }

static double wrapd(double d, double L) {
    if (d > 0.5 * L) d -= L;
    else if (d < -0.5 * L) d += L;
    return d;
}

int mps_rsa(int64_t n, const double *radii, const double *box, uint64_t seed, int64_t max_tries, double *x) {
    double rmax = 0.0, rmin = 1e300;
    for (int64_t i = 0; i < n; ++i) {
        if (radii[i] > rmax) rmax = radii[i];
        if (radii[i] < rmin) rmin = radii[i];
    }
    int nc[3];
    double cw[3];
    for (int d = 0; d < 3; ++d) {
        nc[d] = (int)floor(box[d] / (2.0 * rmax));
        if (nc[d] < 3) nc[d] = 3;
        cw[d] = box[d] / nc[d];
    }
    double ratio = cw[0] / (2.0 * rmin);
    int cap = (int)ceil((ratio + 1.0) * (ratio + 1.0) * (ratio + 1.0)) + 2;
    int64_t ncells = (int64_t)nc[0] * nc[1] * nc[2];
    int32_t *cells = (int32_t *)malloc(sizeof(int32_t) * ncells * cap);
    int32_t *fill = (int32_t *)calloc(ncells, sizeof(int32_t));
    if (!cells || !fill) {
        free(cells);
        free(fill);
        return 2;
    }
    rng_t g;
    uint64_t z = seed;
    for (int k = 0; k < 4; ++k) g.s[k] = splitmix(&z);
    int rc = 0;
    for (int64_t i = 0; i < n && !rc; ++i) {
        int64_t t;
        for (t = 0; t < max_tries; ++t) {
            double p[3];
            int c[3];
            for (int d = 0; d < 3; ++d) {
                p[d] = uniform(&g) * box[d];
                c[d] = (int)(p[d] / cw[d]);
                if (c[d] >= nc[d]) c[d] = nc[d] - 1;
            }
            int ok = 1;
            for (int a = -1; a <= 1 && ok; ++a)
                for (int b = -1; b <= 1 && ok; ++b)
                    for (int e = -1; e <= 1 && ok; ++e) {
                        int cx = (c[0] + a + nc[0]) % nc[0];
                        int cy = (c[1] + b + nc[1]) % nc[1];
                        int cz = (c[2] + e + nc[2]) % nc[2];
                        int64_t cell = ((int64_t)cz * nc[1] + cy) * nc[0] + cx;
                        for (int s = 0; s < fill[cell]; ++s) {
                            int32_t j = cells[cell * cap + s];
                            double dx = wrapd(p[0] - x[3 * j], box[0]);
                            double dy = wrapd(p[1] - x[3 * j + 1], box[1]);
                            double dz = wrapd(p[2] - x[3 * j + 2], box[2]);
                            double cd = radii[i] + radii[j];
                            if (dx * dx + dy * dy + dz * dz < cd * cd) {
                                ok = 0;
                                break;
                            }
                        }
                    }
            if (ok) {
                int64_t cell = ((int64_t)c[2] * nc[1] + c[1]) * nc[0] + c[0];
                if (fill[cell] >= cap) {
                    rc = 3;
                    break;
                }
                cells[cell * cap + fill[cell]++] = (int32_t)i;
                x[3 * i] = p[0];
                x[3 * i + 1] = p[1];
                x[3 * i + 2] = p[2];
                break;
            }
        }
        if (!rc && t == max_tries) rc = 1;
    }
    free(cells);
    free(fill);
    return rc;
}
