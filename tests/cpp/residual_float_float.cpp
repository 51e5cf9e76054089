// Host restatement of the residual row arithmetic of k_solve.cu (float-float:
// Dot2 of Ogita, Rump and Oishi; TwoSum; TwoProduct by a fused multiply-add)
// against plain double arithmetic, over random rows that reach every branch of
// the projection. Prints the largest per-row error of phi relative to the
// row's scale and the largest relative error of the summed phi^2 and lambda^2.
// Built with -ffp-contract=off so that every operation rounds once, as on the
// device (--fmad=false).
#include <cmath>
#include <cstdio>
#include <random>
struct FF { float hi, lo; };
static FF two_sum(float a, float b) { float s = a + b; float z = s - a; return {s, (a - (s - z)) + (b - z)}; }
static FF fast_two_sum(float a, float b) { float s = a + b; return {s, b - (s - a)}; }
static FF two_prod(float a, float b) { float p = a * b; return {p, std::fma(a, b, -p)}; }
static FF ff_norm(FF a) { return two_sum(a.hi, a.lo); }
static bool ff_less(FF a, FF b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
static FF ff_add(FF a, FF b) { FF s = two_sum(a.hi, b.hi); return fast_two_sum(s.hi, s.lo + (a.lo + b.lo)); }
static FF ff_sq(FF a) { FF p = two_prod(a.hi, a.hi); return fast_two_sum(p.hi, p.lo + 2.0f * (a.hi * a.lo)); }
int main() {
    std::mt19937 g(1);
    std::uniform_real_distribution<float> U(-1, 1);
    double worst = 0, worst_l = 0;
    int branches[5] = {0};
    for (int trial = 0; trial < 200; ++trial) {
        FF s2{0, 0}, l2{0, 0};
        double S2 = 0, L2 = 0;
        for (int row = 0; row < 300; ++row) {
            float J[12], dv[12];
            for (int k = 0; k < 12; ++k) { J[k] = U(g) * 2; dv[k] = U(g) * 0.5f; }
            float rhs = U(g), r = std::fabs(U(g)) + 0.1f, lam = U(g) * 0.3f, ln = std::fabs(U(g)) * 0.3f, mu = 0.5f;
            bool fr = row % 3 != 0;
            if (!fr) lam = std::fabs(lam);
            // near-converged rows: make J dv + rhs small
            if (row % 2) { double d = 0; for (int k = 0; k < 12; ++k) d += double(J[k]) * dv[k]; rhs = float(-d + 1e-6 * U(g)); }
            // double reference
            double d = 0; for (int k = 0; k < 12; ++k) d += double(J[k]) * double(dv[k]); d += rhs;
            double x = lam - double(r) * d, p;
            if (!fr) p = x > 0 ? x : 0; else { double mx = double(mu) * ln; p = x < -mx ? -mx : (x > mx ? mx : x); }
            double phi = lam - p; S2 += phi * phi; L2 += double(lam) * lam;
            // float-float
            float ds = 0, dc = 0;
            for (int k = 0; k < 12; ++k) { FF pp = two_prod(J[k], dv[k]); FF t = two_sum(ds, pp.hi); ds = t.hi; dc = dc + (t.lo + pp.lo); }
            { FF t = two_sum(ds, rhs); ds = t.hi; dc = dc + (t.lo + 0.0f); }
            FF D = two_sum(ds, dc);
            FF rd = two_prod(r, D.hi); rd = fast_two_sum(rd.hi, rd.lo + r * D.lo);
            FF X = two_sum(lam, -rd.hi); X = ff_norm(FF{X.hi, X.lo - rd.lo});
            FF ph = rd; int br = 0;
            if (!fr) { if (!(X.hi > 0 || (X.hi == 0 && X.lo > 0))) { ph = FF{lam, 0}; br = 1; } }
            else {
                FF mx = two_prod(mu, ln);
                if (ff_less(X, FF{-mx.hi, -mx.lo})) { FF t = two_sum(lam, mx.hi); ph = ff_norm(FF{t.hi, t.lo + mx.lo}); br = 2; }
                else if (ff_less(mx, X)) { FF t = two_sum(lam, -mx.hi); ph = ff_norm(FF{t.hi, t.lo - mx.lo}); br = 3; }
                else br = 4;
            }
            branches[br]++;
            double phf = double(ph.hi) + ph.lo;
            double scale = std::fabs(double(lam)) + std::fabs(double(r) * d) + double(r) * 3.0 + std::fabs(double(mu) * ln); double e = std::fabs(phf - phi) / scale;
            if (e > worst) worst = e;
            s2 = ff_add(s2, ff_sq(ph)); l2 = ff_add(l2, two_prod(lam, lam));
        }
        double a = double(s2.hi) + s2.lo, b = double(l2.hi) + l2.lo;
        worst_l = std::fmax(worst_l, std::fabs(a - S2) / S2);
        worst_l = std::fmax(worst_l, std::fabs(b - L2) / L2);
    }
    printf("worst per-row phi err / row scale %.3e, worst sum rel err %.3e; branches keep/zero/-mx/+mx/inside %d %d %d %d %d\n",
           worst, worst_l, branches[0], branches[1], branches[2], branches[3], branches[4]);
}
