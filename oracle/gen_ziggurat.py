"""Generate the ziggurat tables for the standard normal sampler.

G. Marsaglia and W. W. Tsang, "The Ziggurat Method for Generating Random
Variables", J. Stat. Software 5(8), 2000: N = 256 layers of equal area v under
f(x) = exp(-x^2/2), x >= 0, with the base layer ending at R (the tail beyond R
is sampled by Marsaglia's exponential method); R and v are the paper's
256-layer values.  Index and value come from separate bits of one 32-bit word
(index: low 8 bits; value: the signed top 24 bits), avoiding the index/value
correlation Doornik (2005) noted in the original.  With 256 layers the fast
test accepts 98.5 % of draws (97.2 % with 128).

Layer i (1..255) is the rectangle [0, x_i] x [f(x_i), f(x_{i+1})] with
x_1 = R > x_2 > ... > x_256 = 0; layer 0 is [0, v/f(R)] x [0, f(R)] plus the
tail.  Tables, with S = 2^23 the magnitude range of the signed value:
K[i] = floor(S * x_{i+1}/x_i) (K[0] = floor(S R f(R)/v)), W[i] = x_i / S
(W[0] = v/f(R)/S), F[i] = f(x_i) (F[0] = f(R), F[256] = 1).  A draw
z = hz*W[iz] with |hz| < K[iz] lies in the part of the layer under the curve
and is accepted at once.

Writes oracle/tm_zig_table.inc (used by the oracle) and
trophic_maelstorm_gb300/csrc/tm_zig_table.cuh (used by the kernels) with the
same literals.

    python oracle/gen_ziggurat.py
"""
import math
import os

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
N = 256
BITS = 8                      # log2(N): index bits of the word
S = 2 ** (31 - BITS)          # magnitude range of the signed value
R = 3.6541528853610088
V = 4.92867323399e-3


def tables():
    f = lambda x: math.exp(-0.5 * x * x)
    x = [0.0] * (N + 1)
    x[1] = R
    for i in range(1, N - 1):
        x[i + 1] = math.sqrt(-2.0 * math.log(f(x[i]) + V / x[i]))
    x[N] = 0.0
    xt0 = V / f(R)
    K = [0] * N
    W = [0.0] * N
    F = [0.0] * (N + 1)
    K[0] = int(math.floor(S * R / xt0))
    W[0] = xt0 / S
    F[0] = f(R)
    for i in range(1, N):
        K[i] = int(math.floor(S * x[i + 1] / x[i]))
        W[i] = x[i] / S
        F[i] = f(x[i])
    F[N] = 1.0
    return K, W, F, x


def emit():
    K, W, F, x = tables()
    kl = ", ".join(f"{k}u" for k in K)
    wl = ", ".join(float(w).hex() for w in W)
    fl = ", ".join(float(v).hex() for v in F)
    common = (f"/* generated by oracle/gen_ziggurat.py: ziggurat for the standard normal\n"
              f" * (Marsaglia & Tsang 2000), {N} layers, R = {R}, v = {V} */\n")
    with open(os.path.join(HERE, "tm_zig_table.inc"), "w") as fh:
        fh.write(common)
        fh.write(f"#define TMO_ZIG_R {float(R).hex()}\n#define TMO_ZIG_BITS {BITS}\n")
        fh.write(f"static const uint32_t tmo_zig_k[{N}] = {{{kl}}};\n")
        fh.write(f"static const double tmo_zig_w[{N}] = {{{wl}}};\n")
        fh.write(f"static const double tmo_zig_f[{N + 1}] = {{{fl}}};\n")
    with open(os.path.join(REPO, "trophic_maelstorm_gb300", "csrc", "tm_zig_table.cuh"), "w") as fh:
        fh.write(common)
        fh.write("#pragma once\n#include <stdint.h>\nnamespace tmg {\n")
        fh.write(f"constexpr int kZigN = {N};\nconstexpr int kZigBits = {BITS};\n")
        fh.write(f"constexpr double kZigR = {float(R).hex()};\n")
        fh.write(f"__device__ const uint32_t kZigK[{N}] = {{{kl}}};\n")
        fh.write(f"__device__ const double kZigW[{N}] = {{{wl}}};\n")
        fh.write(f"__device__ const double kZigF[{N + 1}] = {{{fl}}};\n")
        fh.write("}  // namespace tmg\n")


if __name__ == "__main__":
    K, W, F, x = tables()
    print(f"x_{N - 1} =", x[N - 1], f"x_{N} set to 0; f(x_{N - 1})+v/x_{N - 1} =",
          math.exp(-0.5 * x[N - 1] ** 2) + V / x[N - 1])
    print("K[0..3]", K[:4], f"K[{N - 1}]", K[N - 1], "fast-test acceptance", sum(K) / (N * S))
    emit()
