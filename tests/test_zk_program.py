"""The compiled Zernike programs (csrc/rp_zkprog.h) against the device's
memoised recursion (zk_eval in csrc/rp_device.cuh), on the host: both are
compiled from the library's own sources with g++ (FMA contraction off, as
the plain path's translation unit) and must agree bit for bit on every
radial value, for the first 15, 28 and 45 ANSI terms, for z alone and for
z with its gradient, including the slot aliasing of zernike_Rprime_c.  A
key range the reference never reset must leave the distortion to the
recursion (no program)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "raypier_optics_gb300", "csrc")

HARNESS = r'''
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <vector>
#define RP_ZK_SLOTS 48
#define RP_ZK_DEPTH 24
#define RP_ZKOP_WORDS 7
#define RP_ZKPROG_SLOTS 96
static double nan_d() { return NAN; }
using std::abs; using std::isnan;
@MACHINE@
#include "rp_zkprog.h"
static const short *run(const short *p, double r, double *ws) {
    ws[0] = 0.0; ws[1] = 1.0;
    const short *o = p + 3;
    for (int j = 0; j < p[0]; j++, o += RP_ZKOP_WORDS) {
        const double a = ws[o[2]], b = ws[o[3]], c = ws[o[4]];
        double v;
        if (o[1] == 0) v = r * (a + b) - c;
        else if (o[1] == 1) v = (a + b) + r * (c + ws[o[5]]) - ws[o[6]];
        else v = (a + b) - c;
        ws[o[0]] = v;
    }
    return o;
}
// The polynomial table (rp::zkp) against the program: z, dz/dx, dz/dy of
// ZernikeDistortion.z_offset_c / z_offset_and_gradient_c with the program's
// radial values, over random points and coefficients; prints the largest
// difference relative to the largest |value|.
static int poly_check(int J) {
    std::mt19937_64 g(7);
    std::normal_distribution<double> Nrm(0.0, 1.0);
    std::uniform_real_distribution<double> U(-1.3, 1.3);
    std::vector<double> c;
    int kmax = 0;
    for (int j = 0; j < J; j++) {
        int n = (int)std::ceil((-3 + std::sqrt(9 + 8.0 * j)) / 2), m = 2 * j - n * (n + 2), h = n / 2;
        int k = h * (h + 1) + abs(m);
        if (k + 1 > kmax) kmax = k + 1;
        double row[5] = {(double)j, (double)n, (double)m, (double)k, Nrm(g)};
        c.insert(c.end(), row, row + 5);
    }
    std::vector<short> pz, pg;
    if (!rp::zk_compile(J, kmax, c.data(), false, pz) || !rp::zk_compile(J, kmax, c.data(), true, pg)) return 3;
    rp::zkp::Table t;
    if (!rp::zkp::build(J, 2.0, c.data(), pz, pg, t)) return 4;
    double worst = 0.0, scale = 0.0;
    for (int s = 0; s < 4000; s++) {
        const double X = U(g) * 2.0, Y = U(g) * 2.0, x = X / 2.0, y = Y / 2.0;
        const double r = std::sqrt(x * x + y * y), th = std::atan2(y, x), ct = x / r, st = y / r;
        double w[RP_ZKPROG_SLOTS];
        const short *rz = run(pz.data(), r, w);
        double z = 0.0;
        for (int i = 0; i < J; i++) {
            const int n = (int)c[5 * i + 1], m = (int)c[5 * i + 2];
            const double N = (m == 0 ? std::sqrt(n + 1.0) : std::sqrt(2.0 * (n + 1))) * c[5 * i + 4];
            z += N * w[rz[i]] * (m >= 0 ? std::cos(m * th) : -std::sin(m * th));
        }
        const short *rg = run(pg.data(), r, w);
        double zg = 0.0, zx = 0.0, zy = 0.0;
        for (int i = 0; i < J; i++) {
            const int n = (int)c[5 * i + 1], m = (int)c[5 * i + 2];
            const double N = (m == 0 ? std::sqrt(n + 1.0) : std::sqrt(2.0 * (n + 1))) * c[5 * i + 4];
            const double PH = m >= 0 ? std::cos(m * th) : -std::sin(m * th);
            const double PHp = m >= 0 ? -m * std::sin(m * th) : -m * std::cos(m * th);
            const double R = w[rg[3 * i]], Rp = w[rg[3 * i + 1]], Rr = w[rg[3 * i + 2]];
            zg += N * R * PH;
            zx += N * (Rp * ct * PH + Rr * (-st) * PHp);
            zy += N * (Rp * st * PH + Rr * ct * PHp);
        }
        zx /= 2.0;
        zy /= 2.0;
        // the table: ascending |m| groups, Horner in r
        double tz = 0.0, tg = 0.0, tx = 0.0, ty = 0.0;
        for (const auto &gr : t.groups) {
            const double A = gr.kind ? std::sin(gr.m * th) : std::cos(gr.m * th);
            const double Ad = gr.kind ? gr.m * std::cos(gr.m * th) : -gr.m * std::sin(gr.m * th);
            auto ev = [&](const rp::zkp::Poly &p) { double v = 0.0; for (int k = t.stride - 1; k >= 0; k--) v = v * r + p.c[k]; return v; };
            tz += ev(gr.pz) * A;
            tg += ev(gr.g) * A;
            tx += (ev(gr.q) * ct * A - ev(gr.w) * st * Ad) / 2.0;
            ty += (ev(gr.q) * st * A + ev(gr.w) * ct * Ad) / 2.0;
        }
        for (double v : {z, zg, zx, zy}) scale = std::max(scale, std::fabs(v));
        worst = std::max(worst, std::max(std::max(std::fabs(tz - z), std::fabs(tg - zg)),
                                         std::max(std::fabs(tx - zx), std::fabs(ty - zy))));
    }
    printf("%.3e %d\n", worst / scale, (int)t.groups.size());
    return 0;
}
int main(int argc, char **argv) {
    if (argc > 2 && !strcmp(argv[1], "poly")) return poly_check(atoi(argv[2]));
    const int J = atoi(argv[1]);
    std::vector<double> c;
    int kmax = 0;
    for (int j = 0; j < J; j++) {  // ANSI j -> n, m; key (n/2)(n/2+1) + |m|
        int n = (int)std::ceil((-3 + std::sqrt(9 + 8.0 * j)) / 2), m = 2 * j - n * (n + 2), h = n / 2;
        int k = h * (h + 1) + abs(m);
        if (k + 1 > kmax) kmax = k + 1;
        double row[5] = {(double)j, (double)n, (double)m, (double)k, 1.0};
        c.insert(c.end(), row, row + 5);
    }
    if (argc > 2) kmax = atoi(argv[2]);
    std::mt19937_64 g(1);
    std::uniform_real_distribution<double> U(0.0, 1.5);
    long bad = 0, compiled = 0;
    for (int grad = 0; grad < 2; grad++) {
        std::vector<short> p;
        if (!rp::zk_compile(J, kmax, c.data(), grad == 1, p)) continue;
        compiled++;
        for (int t = 0; t < 2000; t++) {
            const double r = U(g);
            double ws[3][RP_ZK_SLOTS], w2[RP_ZKPROG_SLOTS];
            unsigned err = 0;
            for (int f = 0; f < 3; f++)
                for (int i = 0; i < RP_ZK_SLOTS; i++) ws[f][i] = (f < (grad ? 3 : 1) && i < kmax) ? NAN : 7.0;
            if (!grad) ws[0][0] = 1.0;
            const short *res = run(p.data(), r, w2);
            for (int i = 0; i < J; i++)
                for (int f = 0; f < (grad ? 3 : 1); f++) {
                    const double a = zk_eval(f, (int)c[5 * i + 3], (int)c[5 * i + 1], abs((int)c[5 * i + 2]), r, ws, &err);
                    const double b = w2[res[(grad ? 3 : 1) * i + f]];
                    if (memcmp(&a, &b, 8) != 0) bad++;
                }
            if (err) { printf("recursion error\n"); return 2; }
        }
    }
    printf("%ld %ld\n", compiled, bad);
    return 0;
}
'''


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    src = open(os.path.join(CSRC, "rp_device.cuh")).read()
    start = src.rindex("static __device__", 0, src.index("double zk_eval("))
    machine = src[src.index("struct ZkFrame {"):start]
    body = src[start:]
    body = body[:body.index("\n}\n") + 3]
    body = body.replace("static __device__ __noinline__ ", "static ").replace("static __device__ ", "static ")
    machine += body.replace("atomicOr(err, ERR_ZK_STACK)", "(*err |= 2u)")
    d = tmp_path_factory.mktemp("zk")
    cpp = d / "zk_check.cpp"
    cpp.write_text(HARNESS.replace("@MACHINE@", machine))
    exe = d / "zk_check"
    subprocess.run(["g++", "-O2", "-ffp-contract=off", "-std=c++17", "-I", CSRC, str(cpp), "-o", str(exe)],
                   check=True, capture_output=True)
    return str(exe)


@pytest.mark.parametrize("terms", [15, 28, 45])
def test_program_replays_the_recursion_bit_for_bit(harness, terms):
    out = subprocess.run([harness, str(terms)], check=True, capture_output=True, text=True).stdout.split()
    compiled, bad = int(out[0]), int(out[1])
    assert compiled == 2 and bad == 0


def test_keys_beyond_the_reset_range_stay_with_the_recursion(harness):
    # a workspace reset below the largest key: the reference would read
    # values it never reset, so no program is built
    out = subprocess.run([harness, "15", "5"], check=True, capture_output=True, text=True).stdout.split()
    assert int(out[0]) == 0


@pytest.mark.parametrize("terms", [15, 28, 45])
def test_polynomial_table_equals_the_program(harness, terms):
    """The mixed path's polynomial form of a distortion (rp_zkprog.h, zkp):
    z, dz/dx and dz/dy equal the program's values (aliased slots included)
    to 1e-12 of their size."""
    r = subprocess.run([harness, "poly", str(terms)], capture_output=True, text=True)
    assert r.returncode == 0, r.returncode
    rel, groups = r.stdout.split()
    assert float(rel) < 1e-12 and int(groups) > 0
