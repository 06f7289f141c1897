// rp_zkprog.h -- straight-line programs for the Zernike radial polynomials of
// a distortion (host side, built once per scene).
//
// The reference evaluates R, R' and R/r by recursion memoised in a
// workspace keyed by (function, slot k) (cdistortions.pyx:149-219, 288-316),
// reset before every evaluation; zernike_Rprime_c keys one sub-call with a
// different formula (211), so a slot may be read back for another
// polynomial.  Which slots are filled, and in which order, depends only on
// the distortion's (n, m, k) terms, never on the point: the recursion can be
// run once on the host, each memo miss becoming one operation of a
// straight-line program that the device replays for every point with the
// reference's arithmetic (same operands, same order).  The device falls
// back to the recursion for a distortion this cannot express (a slot key
// outside the workspace, a stack deeper than the device's), which keeps the
// recursion's error reporting.
//
// Program layout (int16): [n_ops, n_slots, n_res], n_ops operations of
// RP_ZKOP_WORDS words {dst, fn, a, b, c, d, e}, then n_res result slots.
// Slot 0 holds 0.0 and slot 1 holds 1.0; operation fn 0 (R) writes
// r * (a + b) - c, fn 1 (R') writes (a + b) + r * (c + d) - e, fn 2 (R/r)
// writes (a + b) - c.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

namespace rp {

struct ZkCompiler {
    int slot[3][RP_ZK_SLOTS];  // dense slot of a filled (fn, k), or -1
    int kmax;                  // keys at or beyond kmax were never reset by the reference
    std::vector<short> ops;
    int n_slots = 2;
    int visits = 0;
    bool ok = true;

    int emit(int fn, int a, int b, int c, int d, int e) {
        if (n_slots >= RP_ZKPROG_SLOTS) {
            ok = false;
            return 0;
        }
        const int dst = n_slots++;
        const short w[RP_ZKOP_WORDS] = {(short)dst, (short)fn, (short)a, (short)b, (short)c, (short)d, (short)e};
        ops.insert(ops.end(), w, w + RP_ZKOP_WORDS);
        return dst;
    }

    // The slot holding function fn of (n, m) at key k, following the device
    // recursion (zk_eval in rp_device.cuh) step for step: base cases, the
    // key check, the memo read, then the sub-calls left to right.
    int eval(int fn, int n, int m, int k, int depth) {
        if (!ok || ++visits > 100000) {
            ok = false;
            return 0;
        }
        if (n < m) return 0;
        if (fn == 0 && n == 0) return 1;
        if (fn == 1 && n == 0) return 0;
        if (k < 0 || k >= kmax) {  // an error, or a key the reference never reset
            ok = false;
            return 0;
        }
        if (slot[fn][k] >= 0) return slot[fn][k];
        if (depth + 1 >= RP_ZK_DEPTH) {
            ok = false;
            return 0;
        }
        int nA = n - 1, mA = std::abs(m - 1), half_n = nA / 2;
        int kA = half_n * (half_n + 1) + std::abs(mA);
        int nB = nA, mB = m + 1;
        int kB = half_n * (half_n + 1) + std::abs(mB);
        int nC = n - 2, mC = m, kC;
        if (fn == 1) {
            kC = (half_n - 1) * half_n + std::abs(mC);  // cdistortions.pyx:211
        } else {
            half_n = nC / 2;
            kC = half_n * (half_n + 1) + std::abs(mC);
        }
        int dst;
        if (fn == 0) {
            const int a = eval(0, nA, mA, kA, depth + 1);
            const int b = eval(0, nB, mB, kB, depth + 1);
            const int c = eval(0, nC, mC, kC, depth + 1);
            dst = emit(0, a, b, c, 0, 0);
        } else if (fn == 1) {
            const int a = eval(0, nA, mA, kA, depth + 1);
            const int b = eval(0, nB, mB, kB, depth + 1);
            const int c = eval(1, nA, mA, kA, depth + 1);
            const int d = eval(1, nB, mB, kB, depth + 1);
            const int e = eval(1, nC, mC, kC, depth + 1);
            dst = emit(1, a, b, c, d, e);
        } else {
            const int a = eval(0, nA, mA, kA, depth + 1);
            const int b = eval(0, nB, mB, kB, depth + 1);
            const int c = eval(2, nC, mC, kC, depth + 1);
            dst = emit(2, a, b, c, 0, 0);
        }
        if (!ok) return 0;
        slot[fn][k] = dst;
        return dst;
    }
};

// Builds the program of a Zernike distortion (coefficient rows of 5
// doubles at `c`: -, n, m, k, value) for z alone (grad = false: z_offset_c,
// whose workspace starts with R(0, 0) = 1 at key 0) or for z and its
// gradient (grad = true: R, R', R/r per term).  Returns false when the
// device must use the recursion instead.
inline bool zk_compile(int n_coefs, int k_max, const double *c, bool grad, std::vector<short> &out) {
    ZkCompiler z;
    z.kmax = k_max < RP_ZK_SLOTS ? k_max : RP_ZK_SLOTS;
    for (int f = 0; f < 3; f++)
        for (int k = 0; k < RP_ZK_SLOTS; k++) z.slot[f][k] = -1;
    if (!grad && z.kmax > 0) z.slot[0][0] = 1;  // ws[0][0] = 1.0
    std::vector<short> res;
    for (int i = 0; i < n_coefs && z.ok; i++) {
        const int n = (int)c[5 * i + 1], m = (int)c[5 * i + 2], k = (int)c[5 * i + 3];
        // the top-level calls take the term's key k, in the device's order
        res.push_back((short)z.eval(0, n, std::abs(m), k, 0));
        if (grad) {
            res.push_back((short)z.eval(1, n, std::abs(m), k, 0));
            res.push_back((short)z.eval(2, n, std::abs(m), k, 0));
        }
    }
    if (!z.ok) return false;
    out.clear();
    out.push_back((short)(z.ops.size() / RP_ZKOP_WORDS));
    out.push_back((short)z.n_slots);
    out.push_back((short)res.size());
    out.insert(out.end(), z.ops.begin(), z.ops.end());
    out.insert(out.end(), res.begin(), res.end());
    return true;
}

// ---- the polynomial form, for the mixed path -------------------------------------
// Every slot of a compiled program is a polynomial in r: slot 0 is 0, slot 1
// is 1, and the three operations add, subtract and multiply by r.  Replaying
// a program on polynomials instead of numbers gives each term's R (and R',
// R/r) as coefficients, aliased slots included, so the mixed kernels can
// evaluate a distortion by Horner's rule in FP32 with no workspace.  The
// terms are summed, with their normalisation and coefficient, per angular
// factor: cos(|m| theta) for m >= 0, sin(|m| theta) for m < 0.
namespace zkp {

constexpr int MAXC = 16;  // coefficients per polynomial (degree <= 15)
struct Poly {
    double c[MAXC] = {};
};

// Replays program p (the layout above) with polynomial operands; false when
// a product would exceed MAXC - 1 in degree.
inline bool replay(const std::vector<short> &p, std::vector<Poly> &res) {
    if (p.size() < 3) return false;
    const int n_ops = p[0], n_slots = p[1], n_res = p[2];
    if ((int)p.size() < 3 + n_ops * RP_ZKOP_WORDS + n_res || n_slots < 2) return false;
    std::vector<Poly> ws((size_t)n_slots);
    ws[1].c[0] = 1.0;
    const short *o = p.data() + 3;
    auto slot = [&](int k) -> const Poly & { return ws[(size_t)k]; };
    for (int j = 0; j < n_ops; j++, o += RP_ZKOP_WORDS) {
        for (int w = 0; w < RP_ZKOP_WORDS; w++)
            if (w != 1 && (o[w] < 0 || o[w] >= n_slots)) return false;
        Poly v;
        const Poly &a = slot(o[2]), &b = slot(o[3]), &c = slot(o[4]);
        if (o[1] == 0) {  // r (a + b) - c
            if (a.c[MAXC - 1] + b.c[MAXC - 1] != 0.0) return false;
            for (int k = 0; k + 1 < MAXC; k++) v.c[k + 1] = a.c[k] + b.c[k];
            for (int k = 0; k < MAXC; k++) v.c[k] -= c.c[k];
        } else if (o[1] == 1) {  // (a + b) + r (c + d) - e
            const Poly &d = slot(o[5]), &e = slot(o[6]);
            if (c.c[MAXC - 1] + d.c[MAXC - 1] != 0.0) return false;
            for (int k = 0; k < MAXC; k++) v.c[k] = a.c[k] + b.c[k] - e.c[k];
            for (int k = 0; k + 1 < MAXC; k++) v.c[k + 1] += c.c[k] + d.c[k];
        } else {  // (a + b) - c
            for (int k = 0; k < MAXC; k++) v.c[k] = a.c[k] + b.c[k] - c.c[k];
        }
        ws[(size_t)o[0]] = v;
    }
    res.clear();
    for (int i = 0; i < n_res; i++) {
        if (o[i] < 0 || o[i] >= n_slots) return false;
        res.push_back(slot(o[i]));
    }
    return true;
}

// The summed polynomials of one angular factor: Pz (z_offset_c's R), G
// (z_offset_and_gradient_c's R), Q (its R') and W (its R / r), each times
// the term's normalisation and coefficient.
struct Group {
    int m = 0, kind = 0;  // |m|; kind 0: cos(|m| theta), 1: sin(|m| theta)
    Poly pz, g, q, w;
};

struct Table {
    std::vector<Group> groups;
    int mmax = 0, stride = 1;
    double unit_radius = 1.0;
};

inline void add_scaled(Poly &dst, const Poly &src, double s) {
    for (int k = 0; k < MAXC; k++) dst.c[k] += s * src.c[k];
}

// The table of a Zernike distortion from its z and z-gradient programs;
// false when either does not replay.
inline bool build(int n_coefs, double unit_radius, const double *c, const std::vector<short> &zprog,
                  const std::vector<short> &gprog, Table &t) {
    std::vector<Poly> rz, rg;
    if (!replay(zprog, rz) || !replay(gprog, rg)) return false;
    if ((int)rz.size() != n_coefs || (int)rg.size() != 3 * n_coefs) return false;
    if (!(unit_radius != 0.0) || !std::isfinite(unit_radius)) return false;
    t = Table();
    t.unit_radius = unit_radius;
    int top = 0;
    for (int i = 0; i < n_coefs; i++) {
        const int n = (int)c[5 * i + 1], m = (int)c[5 * i + 2];
        const double N = (m == 0 ? std::sqrt((double)(n + 1)) : std::sqrt((double)(2 * (n + 1)))) * c[5 * i + 4];
        const int am = std::abs(m), kind = m >= 0 ? 0 : 1;
        Group *g = nullptr;
        for (auto &e : t.groups)
            if (e.m == am && e.kind == kind) g = &e;
        if (!g) {
            t.groups.push_back(Group());
            g = &t.groups.back();
            g->m = am;
            g->kind = kind;
        }
        add_scaled(g->pz, rz[(size_t)i], N);
        add_scaled(g->g, rg[(size_t)3 * i], N);
        add_scaled(g->q, rg[(size_t)3 * i + 1], N);
        add_scaled(g->w, rg[(size_t)3 * i + 2], N);
        t.mmax = std::max(t.mmax, am);
    }
    // the device steps cos / sin of m theta up from m = 0: ascending |m|
    std::stable_sort(t.groups.begin(), t.groups.end(),
                     [](const Group &a, const Group &b) { return a.m < b.m || (a.m == b.m && a.kind < b.kind); });
    for (const auto &g : t.groups)
        for (const Poly *p : {&g.pz, &g.g, &g.q, &g.w})
            for (int k = 0; k < MAXC; k++)
                if (p->c[k] != 0.0) top = std::max(top, k);
    t.stride = top + 1;
    return true;
}

// The words of a table for the device, in double (the FP64 iteration) and
// in float at the same word offsets: n_groups, stride, mmax, 1 / unit
// radius; then per group m, kind, two unused words and the four polynomials
// (stride coefficients each, ascending).  The integers are exact in both.
inline void pack(const Table &t, std::vector<double> &out) {
    out.push_back((double)t.groups.size());
    out.push_back((double)t.stride);
    out.push_back((double)t.mmax);
    out.push_back(1.0 / t.unit_radius);
    for (const auto &g : t.groups) {
        out.push_back((double)g.m);
        out.push_back((double)g.kind);
        out.push_back(0.0);
        out.push_back(0.0);
        for (const Poly *p : {&g.pz, &g.g, &g.q, &g.w})
            for (int k = 0; k < t.stride; k++) out.push_back(p->c[k]);
    }
}

}  // namespace zkp

}  // namespace rp
