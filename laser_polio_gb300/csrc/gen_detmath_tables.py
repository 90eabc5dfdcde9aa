"""Tables of lpg_detmath.h: correctly rounded values from 60-digit decimal
arithmetic (Python's decimal module), printed as C hex-float initialisers.

  log: for j = 0..128, F_j = 1 + j/128 (j < 64) or (1 + j/128) / 2 (j >= 64);
       LOG_HI[j] + LOG_LO[j] = ln F_j (a double-double), INV[j] = 1 / F_j.
  exp: for j = 0..63, EXP_HI[j] + EXP_LO[j] = 2^(j/64).
  lfact: for k = 0..255, LFACT[k] = ln k! (Poisson inversion from the mode).

python gen_detmath_tables.py > /dev/stdout   (paste into lpg_detmath.h)
"""

from decimal import Decimal, getcontext

getcontext().prec = 60


def dd(v):
    hi = float(v)
    lo = float(v - Decimal(hi))
    return hi, lo


def table(name, vals):
    body = ",\n".join("  " + ", ".join(x.hex() for x in vals[i : i + 4]) for i in range(0, len(vals), 4))
    return f"{name} = {{\n{body}}};"


def main():
    log_hi, log_lo, inv = [], [], []
    for j in range(129):
        f = Decimal(1) + Decimal(j) / Decimal(128)
        if j >= 64:
            f = f / 2
        h, l = dd(f.ln())
        log_hi.append(h)
        log_lo.append(l)
        inv.append(float(Decimal(1) / f))
    exp_hi, exp_lo = [], []
    ln2 = Decimal(2).ln()
    for j in range(64):
        h, l = dd((ln2 * Decimal(j) / Decimal(64)).exp())
        exp_hi.append(h)
        exp_lo.append(l)
    lfact, acc = [], Decimal(0)
    for k in range(256):
        if k >= 2:
            acc += Decimal(k).ln()
        lfact.append(float(acc))
    for name, vals in (("LOG_HI", log_hi), ("LOG_LO", log_lo), ("INV", inv), ("EXP_HI", exp_hi), ("EXP_LO", exp_lo),
                       ("LFACT", lfact)):
        print(table(f"LPG_TAB_{name}[{len(vals)}]", vals))


if __name__ == "__main__":
    main()
