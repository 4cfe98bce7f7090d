/* Conservativeness of the blend's per-block cull, on the CPU.
 *
 * A C restatement of block_mask<kSlabs>() and of the per-pixel p2 of
 * torpedo_gb300/csrc/blend.cu (same float operations, fmaf for the fused
 * ones, compiled with -ffp-contract=off). For random entries near one tile,
 * including thin, rotated, huge and near-threshold ones, every pixel of every
 * 8-wide block that the exact per-pixel rule keeps (p2 <= 0 and p2 >= thr)
 * must lie in a block whose mask bit is set. The GPU's sqrt.approx and
 * rcp.approx results are stood in for by correctly rounded ones nudged by
 * -/+ 2^-22 relative, both ways.
 *
 * usage: cull_mask_check <entries> <seed>; prints "violations N visits V truth T"
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

static const float kLog2e = 1.4426950408889634f;
static double g_nudge = 0.0;  /* relative nudge of the approximate sqrt / reciprocal */

static float sqrt_approx(float x) { return (float)(sqrtf(x) * (1.0 + g_nudge)); }
static float rcp_approx(float x) { return (float)((1.0f / x) * (1.0 - g_nudge)); }

/* block_mask<kSlabs> of blend.cu: bit 2k + c for block row k, block column c */
static unsigned block_mask(int slabs, float cx, float cy, float qa, float qb, float qc, float thr, float ox, float oy) {
    const float rows = 16.0f / (float)slabs;
    if (!(thr <= 0.0f)) return 0u;
    const float a = -qa, c = -qc, b = -0.5f * qb;
    const float w = b * b;
    const float det = fmaf(a, c, -w) + fmaf(-b, b, w);
    if (!(a > 0.0f && c > 0.0f && det > 0.0f)) return 0xFFu;
    const float inv_det = rcp_approx(det), inv_a = rcp_approx(a);
    const float R = -thr * (1.0f + 4e-3f + 1e-5f * (a * c * inv_det)) + 4e-3f;
    const float hx = sqrt_approx(c * R * inv_det), hy = sqrt_approx(a * R * inv_det);
    const float dyr = -b * hx * rcp_approx(c);
    const float aR = a * R;
    const float wx = 0.02f + 1e-4f * hx;
    unsigned m = 0;
    for (int k = 0; k < slabs; ++k) {
        const float y0 = oy + rows * (float)k;
        float dlo = cy - (y0 + (rows - 1.0f)) - 0.01f, dhi = cy - y0 + 0.01f;
        if (dhi < -hy || dlo > hy) continue;
        dlo = fmaxf(dlo, -hy);
        dhi = fminf(dhi, hy);
        const float s0 = sqrt_approx(fmaxf(fmaf(-det, dlo * dlo, aR), 0.0f));
        const float s1 = sqrt_approx(fmaxf(fmaf(-det, dhi * dhi, aR), 0.0f));
        float xmax = fmaxf((-b * dlo + s0) * inv_a, (-b * dhi + s1) * inv_a);
        float xmin = fminf((-b * dlo - s0) * inv_a, (-b * dhi - s1) * inv_a);
        if (dyr >= dlo && dyr <= dhi) xmax = hx;
        if (-dyr >= dlo && -dyr <= dhi) xmin = -hx;
        const float pxlo = cx - xmax - wx, pxhi = cx - xmin + wx;
        if (pxlo <= ox + 7.0f && pxhi >= ox) m |= 1u << (2 * k);
        if (pxlo <= ox + 15.0f && pxhi >= ox + 8.0f) m |= 2u << (2 * k);
    }
    return m;
}

/* the per-pixel p2 of the blend: dx = x - px, dy = y - py,
 * p2 = fma(fma(qb, dy, qa dx), dx, (qc dy) dy) */
static float pair_p2(float x, float y, float qa, float qb, float qc, float px, float py) {
    const float dx = x - px, dy = y - py;
    return fmaf(fmaf(qb, dy, qa * dx), dx, (qc * dy) * dy);
}

static uint64_t st;
static double urand(void) {
    st ^= st << 13; st ^= st >> 7; st ^= st << 17;
    return (double)(st >> 11) * (1.0 / 9007199254740992.0);
}

int main(int argc, char** argv) {
    const long n = argc > 1 ? atol(argv[1]) : 200000;
    st = 88172645463325252ull ^ (uint64_t)(argc > 2 ? atol(argv[2]) : 1);
    long viol = 0, visits = 0, truth = 0;
    for (long it = 0; it < n; ++it) {
        const float ox = 16.0f * (int)(urand() * 240), oy = 16.0f * (int)(urand() * 135);
        /* covariance eigenvalues 0.3 .. 3e5 px^2 (plus the 0.3 dilation), any angle */
        const double l1 = exp(log(0.3) + urand() * (log(3e5) - log(0.3)));
        const double l2 = exp(log(0.3) + urand() * (log(3e5) - log(0.3)));
        const double th = urand() * 3.14159265358979, cs = cos(th), sn = sin(th);
        const double sxx = l1 * cs * cs + l2 * sn * sn + 0.3, syy = l1 * sn * sn + l2 * cs * cs + 0.3;
        const double sxy = (l1 - l2) * cs * sn, det = sxx * syy - sxy * sxy;
        const float A = (float)(syy / det), B = (float)(-sxy / det), C = (float)(sxx / det);
        const double rad = 3.0 * sqrt(fmax(l1, l2) + 0.3);
        const float x = ox + 8 + (float)((urand() * 2 - 1) * fmin(rad, 3000));
        const float y = oy + 8 + (float)((urand() * 2 - 1) * fmin(rad, 3000));
        const float o = (float)(urand() < 0.5 ? (1.0 / 255) * (1 + urand() * 0.01) : urand());
        const float thr = o > 0.0f ? -log2f(255.0f * o) : INFINITY;
        const float qa = -0.5f * kLog2e * A, qb = -kLog2e * B, qc = -0.5f * kLog2e * C;
        for (int pass = 0; pass < 2; ++pass) {
            g_nudge = pass ? 2.4e-7 : -2.4e-7;
            for (int slabs = 2; slabs <= 4; slabs += 2) {
                const unsigned m = block_mask(slabs, x, y, qa, qb, qc, thr, ox, oy);
                const int rows = 16 / slabs;
                for (int blk = 0; blk < 2 * slabs; ++blk) {
                    const float bx = ox + 8 * (blk & 1), by = oy + rows * (blk >> 1);
                    int kept = 0;
                    for (int ly = 0; ly < rows && !kept; ++ly)
                        for (int lx = 0; lx < 8; ++lx) {
                            const float p2 = pair_p2(x, y, qa, qb, qc, bx + lx, by + ly);
                            if (!(p2 > 0.0f || p2 < thr)) { kept = 1; break; }
                        }
                    truth += kept;
                    visits += (m >> blk) & 1u;
                    if (kept && !((m >> blk) & 1u)) ++viol;
                }
            }
        }
    }
    printf("violations %ld visits %ld truth %ld\n", viol, visits, truth);
    return viol != 0;
}
