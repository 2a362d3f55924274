"""Write rot_coeffs.cuh: coefficients of the real-harmonic rotation recursion.

The rotation matrix D^l of the real spherical harmonics (order m = -l..l)
is built from D^1 and D^(l-1) with the recursion of Ivanic and Ruedenberg
(J. Phys. Chem. 100, 6342 (1996); erratum 102, 9099 (1998)):

    D^l[m][n] = u U + v V + w W,

where U, V, W are sums of products P(i, a, b) of one D^1 entry and one
D^(l-1) entry.  For every (l, m, n) with l = 2, 3 this script stores the
five scalar weights multiplying P_U, P_V1, P_V2, P_W1, P_W2 (zeros where a
term is absent).  Run: python gen_rot_coeffs.py > rot_coeffs.cuh
"""
import math


def weights(l, m, n):
    d = 1 if m == 0 else 0
    denom = (2 * l) * (2 * l - 1) if abs(n) == l else (l + n) * (l - n)
    u = math.sqrt((l + m) * (l - m) / denom)
    v = 0.5 * math.sqrt((1 + d) * (l + abs(m) - 1) * (l + abs(m)) / denom) * (1 - 2 * d)
    w = -0.5 * math.sqrt(max(0, (l - abs(m) - 1) * (l - abs(m))) / denom) * (1 - d)
    # V = cv1 * P(+1, ...) + cv2 * P(-1, ...);  W = cw1 * P(+1, ...) + cw2 * P(-1, ...)
    if m == 0:
        cv1, cv2 = 1.0, 1.0
        cw1, cw2 = 0.0, 0.0
    elif m > 0:
        dd = 1 if m == 1 else 0
        cv1, cv2 = math.sqrt(1 + dd), -(1 - dd)
        cw1, cw2 = 1.0, 1.0
    else:
        dd = 1 if m == -1 else 0
        cv1, cv2 = (1 - dd), math.sqrt(1 + dd)
        cw1, cw2 = 1.0, -1.0
    return [u, v * cv1, v * cv2, w * cw1, w * cw2]


def main():
    print("// Generated by gen_rot_coeffs.py -- weights of the real-harmonic rotation recursion.")
    print("// Entry (l, m, n) at SKN_ROT_OFF[l] + (m + l) * (2l + 1) + (n + l); five weights each:")
    print("// P_U, P_V(+1), P_V(-1), P_W(+1), P_W(-1).")
    print("#pragma once")
    rows = []
    off = {}
    cnt = 0
    for l in (2, 3):
        off[l] = cnt
        for m in range(-l, l + 1):
            for n in range(-l, l + 1):
                rows.append(weights(l, m, n))
                cnt += 1
    print(f"#define SKN_ROT_NENT {cnt}")
    print(f"static __device__ const int SKN_ROT_OFF[4] = {{0, 0, {off[2]}, {off[3]}}};")
    print("static __device__ const double SKN_ROT_W[SKN_ROT_NENT * 5] = {")
    for r in rows:
        print("  " + ", ".join(repr(float(x)) for x in r) + ",")
    print("};")


if __name__ == "__main__":
    main()
