/*
 * CPU oracle of the "siddon" projector model, in double precision.
 * TEST INFRASTRUCTURE ONLY: the product never links this file.
 *
 * The reference ships no such model (only projector-parallel-joseph.cl), so
 * parity is unpinned by the reference: this restatement is pinned instead by
 * an analytic known answer (the projection of a uniform image is the chord
 * of each ray through the image square, oracle_siddon_chord) and by the
 * adjointness of its two halves.
 *
 * Geometry (the reference backprojector's, projector-parallel-joseph.cl:
 * 174-195): pixel (i, j) covers X in [i - n/2, i + 1 - n/2] and
 * Y in [j - n/2, j + 1 - n/2]; bin k of angle theta is the line
 * X cos - Y sin + axis = k + 0.5.
 *   forward  sino[a][k] = sum_pixels L(ray, pixel) vol[pixel], per ray by
 *            walking slabs (rows when |cos| >= |sin|, else columns);
 *   backward vol[pixel] = sum_a sum_k L(ray, pixel) sino[a][k], per pixel
 *            from the chord of a line through a unit square (a trapezoid in
 *            the line's offset from the pixel centre).
 */
#include <math.h>
#include <stddef.h>

void oracle_siddon_forward(unsigned int n, unsigned int n_angles, const float *sinv, const float *cosv, float axis,
                           const float *vol, double *sino)
{
    const double half = 0.5 * n;
#pragma omp parallel for schedule(static)
    for (long q = 0; q < (long) n_angles * n; ++q) {
        const unsigned int a = (unsigned int) (q / n), k = (unsigned int) (q % n);
        /* the line, with its normal scaled to unit length (the float LUT's
         * sin^2 + cos^2 is not exactly 1): lengths are Euclidean */
        const double r = sqrt((double) sinv[a] * sinv[a] + (double) cosv[a] * cosv[a]);
        const double sn = sinv[a] / r, cs = cosv[a] / r;
        const double u0 = (k + 0.5 - (double) axis) / r;
        double sum = 0.0;
        const int rows = fabs(cs) >= fabs(sn);
        const double len = rows ? 1.0 / fabs(cs) : 1.0 / fabs(sn);
        for (unsigned int m = 0; m < n; ++m) {
            /* coordinate across the slab at its two edges */
            const double e0 = m - half, e1 = e0 + 1.0;
            const double pa = rows ? (u0 + e0 * sn) / cs + half : (e0 * cs - u0) / sn + half;
            const double pb = rows ? (u0 + e1 * sn) / cs + half : (e1 * cs - u0) / sn + half;
            const double lo = pa < pb ? pa : pb, hi = pa < pb ? pb : pa;
            const double c0f = floor(lo);
            const long c0 = (long) c0f;
            const double f = hi > c0f + 1.0 ? (c0f + 1.0 - lo) / (hi - lo) : 1.0;
            for (int h = 0; h < 2; ++h) {
                const long c = c0 + h;
                const double part = h ? 1.0 - f : f;
                if (part <= 0.0 || c < 0 || c >= (long) n)
                    continue;
                const size_t idx = rows ? (size_t) m * n + (size_t) c : (size_t) c * n + m;
                sum += len * part * (double) vol[idx];
            }
        }
        sino[q] = sum;
    }
}

void oracle_siddon_backward(unsigned int n, unsigned int n_angles, const float *sinv, const float *cosv,
                            float axis, const float *sino, double *vol)
{
    const double half = 0.5 * n;
#pragma omp parallel for schedule(static)
    for (long q = 0; q < (long) n * n; ++q) {
        const unsigned int j = (unsigned int) (q / n), i = (unsigned int) (q % n);
        const double X = i + 0.5 - half, Y = j + 0.5 - half;
        double v = 0.0;
        for (unsigned int a = 0; a < n_angles; ++a) {
            const double r = sqrt((double) sinv[a] * sinv[a] + (double) cosv[a] * cosv[a]);
            const double sn = sinv[a] / r, cs = cosv[a] / r;
            const double ca = fabs(cs), sa = fabs(sn);
            /* bin coordinate of the pixel centre; distances along the unit normal are (u - uc) / r */
            const double uc = (X * cs - Y * sn) * r + axis;
            const double w = 0.5 * (ca + sa), p = 0.5 * fabs(ca - sa);
            const double h = 1.0 / (ca > sa ? ca : sa);
            long k0 = (long) ceil(uc - w * r - 0.5), k1 = (long) floor(uc + w * r - 0.5);
            k0 = k0 < 0 ? 0 : k0;
            k1 = k1 > (long) n - 1 ? (long) n - 1 : k1;
            for (long k = k0; k <= k1; ++k) {
                const double d = fabs(k + 0.5 - uc) / r;
                const double L = d <= p ? h : (d < w ? (w - d) / (ca * sa) : 0.0);
                v += L * (double) sino[(size_t) a * n + (size_t) k];
            }
        }
        vol[q] = v;
    }
}

/* Chord of bin k's line through the image square [-n/2, n/2]^2 (clipping
 * the line's parameter to the two slabs): the projection of an image of ones. */
double oracle_siddon_chord(unsigned int n, float sinv, float cosv, float axis, unsigned int k)
{
    const double r = sqrt((double) sinv * sinv + (double) cosv * cosv);
    const double half = 0.5 * n, sn = sinv / r, cs = cosv / r;
    const double u0 = (k + 0.5 - (double) axis) / r;
    /* the line: P(t) = u0 * (cs, -sn) + t * (sn, cs) */
    const double px = u0 * cs, py = -u0 * sn, dx = sn, dy = cs;
    double t0 = -1e300, t1 = 1e300;
    const double p[2] = {px, py}, dv[2] = {dx, dy};
    for (int c = 0; c < 2; ++c) {
        if (fabs(dv[c]) < 1e-300) {
            if (p[c] < -half || p[c] > half)
                return 0.0;
            continue;
        }
        double ta = (-half - p[c]) / dv[c], tb = (half - p[c]) / dv[c];
        if (ta > tb) {
            const double tmp = ta;
            ta = tb;
            tb = tmp;
        }
        t0 = ta > t0 ? ta : t0;
        t1 = tb < t1 ? tb : t1;
    }
    return t1 > t0 ? t1 - t0 : 0.0;
}
