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
#include <cstdint>
#include <cstdlib>
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

}  // namespace rp
