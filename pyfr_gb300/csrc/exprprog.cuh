// Postfix programs of boundary values and source terms, evaluated per
// point.  The host compiles an expression of the point's coordinates, the
// time and (for source terms) the solution into straight-line postfix code
// (pyfr_gb300/bcexpr.py); the opcodes are those of b200_bcop_t in
// pyfrb200.h.
#pragma once

#include <cstdint>

#include "pyfrb200.h"

namespace b200 {

constexpr int EXPR_STACK = 16;
constexpr int EXPR_OP_MAX = 29;

// The value of the program prog[start, start + len) at a point with
// coordinates x, time t and solution u (NULL where the program may not
// read it).  A malformed program, which the host compiler never makes,
// gives NaN instead of leaving the stack.
template <typename T>
__device__ T expr_program(const b200_bcop_t *prog, int start, int len, const T *x, T t,
                          const T *u = nullptr, int nvars = 0) {
    T st[EXPR_STACK];
    int sp = 0;
    const T bad = T(0) / T(0);
    for (int i = start; i < start + len; i++) {
        const int op = prog[i].op;
        if (op < 0 || op > EXPR_OP_MAX) return bad;
        if (op <= 4 || op == 29) {
            if (sp >= EXPR_STACK) return bad;
            T v;
            if (op == 29) {
                const int k = prog[i].pad;
                if (u == nullptr || k < 0 || k >= nvars) return bad;
                v = u[k];
            } else {
                v = op == 0 ? (T)prog[i].val : (op == 4 ? t : x[op - 1]);
            }
            st[sp++] = v;
        } else if (op <= 9 || op >= 24 && op <= 26) {
            if (sp < 2) return bad;
            const T b = st[--sp], a = st[sp - 1];
            T r;
            switch (op) {
            case 5: r = a + b; break;
            case 6: r = a - b; break;
            case 7: r = a * b; break;
            case 8: r = a / b; break;
            case 9: r = pow(a, b); break;
            case 24: r = atan2(a, b); break;
            case 25: r = fmin(a, b); break;
            default: r = fmax(a, b); break;
            }
            st[sp - 1] = r;
        } else {
            if (sp < 1) return bad;
            const T a = st[sp - 1];
            T r;
            switch (op) {
            case 10: r = -a; break;
            case 11: r = sin(a); break;
            case 12: r = cos(a); break;
            case 13: r = tan(a); break;
            case 14: r = exp(a); break;
            case 15: r = log(a); break;
            case 16: r = sqrt(a); break;
            case 17: r = tanh(a); break;
            case 18: r = fabs(a); break;
            case 19: r = asin(a); break;
            case 20: r = acos(a); break;
            case 21: r = atan(a); break;
            case 22: r = sinh(a); break;
            case 23: r = cosh(a); break;
            case 27: r = floor(a); break;
            default: r = ceil(a); break;
            }
            st[sp - 1] = r;
        }
    }
    return sp == 1 ? st[0] : bad;
}

}  // namespace b200
