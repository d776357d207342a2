"""Generate pow_tables.h: the tables of the integer-pipe FP64 pow (pow_int.cuh).

    python hydrofv_gb300/csrc/gpu/gen_pow_tables.py > hydrofv_gb300/csrc/gpu/pow_tables.h

Every entry is a rounded value of an exact mathematical quantity, computed
with 300-bit mpmath arithmetic:

  INV1[i], i = 0..127      round(2^21 / (1 + (2i+1)/256))         first log2 reduction
  LG1[i]                   (21 - log2 INV1[i]) * 2^100              (Q100, unsigned)
  INV2[j+64], j = -64..64  round(2^30 / (1 + j/2^14))             second log2 reduction
  LG2[j+64]                (30 - log2 INV2[j]) * 2^100              (Q100, two's complement)
  EX1[k], k = 0..127       (2^(k/128) - 1) * 2^127                  (Q127)
  EX2[k], k = 0..127       (2^(k/16384) - 1) * 2^127                (Q127)
  INVLN2_HI, INVLN2_LO     2^127 / ln 2 (high and low 64 bits)
  LN2_Q64                  2^64 ln 2
  D2..D6 (Q62)             1 / (k ln 2), the log2(1+r) series coefficients
  INV6_Q64, INV24_Q64      2^64 / 6, 2^64 / 24

128-bit values are emitted as (high, low) 64-bit halves.
"""
import mpmath as mp

mp.mp.prec = 300
M64 = (1 << 64) - 1


def rnd(x):
    return int(mp.nint(x))


def u128(v):
    v &= (1 << 128) - 1
    return f"{{0x{v >> 64:016x}ull, 0x{v & M64:016x}ull}}"


def main():
    out = []
    out.append("/* Generated by gen_pow_tables.py: do not edit. */")
    out.append("#ifndef HYDRO_GPU_POW_TABLES_H")
    out.append("#define HYDRO_GPU_POW_TABLES_H")
    inv1 = [rnd(mp.mpf(2) ** 21 / (1 + mp.mpf(2 * i + 1) / 256)) for i in range(128)]
    lg1 = [rnd((21 - mp.log(v, 2)) * mp.mpf(2) ** 100) for v in inv1]
    inv2 = [rnd(mp.mpf(2) ** 30 / (1 + mp.mpf(j) / 2 ** 14)) for j in range(-64, 65)]
    lg2 = [rnd((30 - mp.log(v, 2)) * mp.mpf(2) ** 100) for v in inv2]
    ex1 = [rnd((mp.mpf(2) ** (mp.mpf(k) / 128) - 1) * mp.mpf(2) ** 127) for k in range(128)]
    ex2 = [rnd((mp.mpf(2) ** (mp.mpf(k) / 16384) - 1) * mp.mpf(2) ** 127) for k in range(128)]
    assert all(0 < v < (1 << 128) for v in lg1)
    assert all(0 <= v < (1 << 127) for v in ex1 + ex2)

    def table(name, vals, fmt):
        out.append(f"#define {name} {{ \\")
        for k in range(0, len(vals), 4):
            chunk = ", ".join(fmt(v) for v in vals[k:k + 4])
            out.append(f"    {chunk}, \\")
        out.append("}")

    table("HYDRO_POW_INV1", inv1, lambda v: f"{v}u")
    table("HYDRO_POW_LG1", lg1, u128)
    table("HYDRO_POW_INV2", inv2, lambda v: f"{v}u")
    table("HYDRO_POW_LG2", lg2, u128)
    table("HYDRO_POW_EX1", ex1, u128)
    table("HYDRO_POW_EX2", ex2, u128)
    ln2 = mp.log(2)
    consts = {
        "HYDRO_POW_INVLN2_HI": rnd(mp.mpf(2) ** 127 / ln2) >> 64,
        "HYDRO_POW_INVLN2_LO": rnd(mp.mpf(2) ** 127 / ln2) & M64,
        "HYDRO_POW_LN2_Q64": rnd(mp.mpf(2) ** 64 * ln2),
        "HYDRO_POW_D2": rnd(mp.mpf(2) ** 62 / (2 * ln2)),
        "HYDRO_POW_D3": rnd(mp.mpf(2) ** 62 / (3 * ln2)),
        "HYDRO_POW_D4": rnd(mp.mpf(2) ** 62 / (4 * ln2)),
        "HYDRO_POW_D5": rnd(mp.mpf(2) ** 62 / (5 * ln2)),
        "HYDRO_POW_D6": rnd(mp.mpf(2) ** 62 / (6 * ln2)),
        "HYDRO_POW_INV6_Q64": rnd(mp.mpf(2) ** 64 / 6),
        "HYDRO_POW_INV24_Q64": rnd(mp.mpf(2) ** 64 / 24),
    }
    for k, v in consts.items():
        assert 0 < v < (1 << 64)
        out.append(f"#define {k} 0x{v:016x}ull")
    out.append("#endif")
    print("\n".join(out))


if __name__ == "__main__":
    main()
