"""Generates dp_asm.cuh: the per-residue update of a register tile of the
banded bit-parallel LCS as one inline-PTX block per (planes, tile width,
carry-in, carry-out) combination.

For every slot m of the tile (one 32-bit word of representative rows):
    x  = row & ~(p0 ^ m0) & ~(p1 ^ m1) ...   one LOP3 per plane
    t  = row + x + carry                    add on the carry flag (add.cc/addc.cc)
    row = t | (row ^ x)                      one LOP3
so the carry of the multi-word addition rides the hardware carry flag from
slot to slot without leaving the flag.  With carry-in, the next column carry
is popped from the top bit of `cw` (add.cc cw, cw, cw); with carry-out, the
final carry is pushed into `ncw` (addc ncw, ncw, ncw) — one instruction each.

Run `python gen_dp_asm.py` after editing; the output is committed.
"""
from pathlib import Path

PLANES = (2, 5)
WIDTHS = tuple(range(1, 33))


def one(P: int, TW: int, cin: bool, cout: bool) -> str:
    # operand numbering: outputs first (row[0..TW-1], then cw, ncw), inputs after
    outs = [f'"+r"(row[{m}])' for m in range(TW)]
    idx_cw = idx_ncw = None
    if cin:
        idx_cw = len(outs)
        outs.append('"+r"(cw)')
    if cout:
        idx_ncw = len(outs)
        outs.append('"+r"(ncw)')
    ins = []
    pl_idx = {}
    for p in range(P):
        for m in range(TW):
            pl_idx[(p, m)] = len(outs) + len(ins)
            ins.append(f'"r"(pl[{p}][{m}])')
    mk_idx = {}
    for p in range(P):
        mk_idx[p] = len(outs) + len(ins)
        ins.append(f'"r"(mk[{p}])')
    lines = ["{", ".reg .u32 a, x, t;"]
    if cin:
        lines.append(f"add.cc.u32 %{idx_cw}, %{idx_cw}, %{idx_cw};")
    for m in range(TW):
        src = f"%{m}"
        for p in range(P):
            dst = "x" if p == P - 1 else "a"
            lines.append(f"lop3.b32 {dst}, {src}, %{pl_idx[(p, m)]}, %{mk_idx[p]}, 0x90;")
            src = "a"
        first = (m == 0 and not cin)
        last_no_out = (m == TW - 1 and not cout)
        op = "add" if first else "addc"
        cc = "" if last_no_out else ".cc"
        lines.append(f"{op}{cc}.u32 t, %{m}, x;")
        lines.append(f"lop3.b32 %{m}, t, %{m}, x, 0xF6;")
    if cout:
        lines.append(f"addc.u32 %{idx_ncw}, %{idx_ncw}, %{idx_ncw};")
    lines.append("}")
    body = "\n".join(f'      "{ln}\\n\\t"' for ln in lines)
    sig = (f"template <>\n__device__ __forceinline__ void dp_tile<{P}, {TW}, {str(cin).lower()}, "
           f"{str(cout).lower()}>(uint32_t (&row)[{TW}], const uint32_t (&pl)[{P}][{TW}], "
           f"const uint32_t (&mk)[{P}], uint32_t &cw, uint32_t &ncw) {{\n")
    unused = []
    if not cin:
        unused.append("cw")
    if not cout:
        unused.append("ncw")
    void = "".join(f"  (void){u};\n" for u in unused)
    return (sig + void + "  asm(\n" + body + "\n      : " + ", ".join(outs) + "\n      : " + ", ".join(ins) +
            ");\n}\n")


def one_eq(TW: int, cin: bool, cout: bool) -> str:
    """DNA tile update from precomputed match words: e[m] is the match word of
    slot m for the column's residue (read from the representative's match
    table), so the match costs one AND instead of one LOP3 per plane:
        x = row & e;  t = row + x + carry;  row = t | (row ^ x)
    three integer instructions per 32 cells."""
    outs = [f'"+r"(row[{m}])' for m in range(TW)]
    idx_cw = idx_ncw = None
    if cin:
        idx_cw = len(outs)
        outs.append('"+r"(cw)')
    if cout:
        idx_ncw = len(outs)
        outs.append('"+r"(ncw)')
    ins = []
    e_idx = {}
    for m in range(TW):
        e_idx[m] = len(outs) + len(ins)
        ins.append(f'"r"(e[{m}])')
    lines = ["{", ".reg .u32 x, t;"]
    if cin:
        lines.append(f"add.cc.u32 %{idx_cw}, %{idx_cw}, %{idx_cw};")
    for m in range(TW):
        lines.append(f"and.b32 x, %{m}, %{e_idx[m]};")
        first = (m == 0 and not cin)
        last_no_out = (m == TW - 1 and not cout)
        op = "add" if first else "addc"
        cc = "" if last_no_out else ".cc"
        lines.append(f"{op}{cc}.u32 t, %{m}, x;")
        lines.append(f"lop3.b32 %{m}, t, %{m}, x, 0xF6;")
    if cout:
        lines.append(f"addc.u32 %{idx_ncw}, %{idx_ncw}, %{idx_ncw};")
    lines.append("}")
    body = "\n".join(f'      "{ln}\\n\\t"' for ln in lines)
    sig = (f"template <>\n__device__ __forceinline__ void dp_tile_eq<{TW}, {str(cin).lower()}, "
           f"{str(cout).lower()}>(uint32_t (&row)[{TW}], const uint32_t (&e)[{TW}], uint32_t &cw, "
           f"uint32_t &ncw) {{\n")
    unused = []
    if not cin:
        unused.append("cw")
    if not cout:
        unused.append("ncw")
    void = "".join(f"  (void){u};\n" for u in unused)
    return (sig + void + "  asm(\n" + body + "\n      : " + ", ".join(outs) + "\n      : " + ", ".join(ins) +
            ");\n}\n")


def one_eqf(TW: int, cin: bool, cout: bool, madc: int) -> str:
    """one_eq with part of the integer work on the FMA pipe: the tile's
    column carry is popped and pushed by multiply-adds with a run-time 1
    (mad.lo.cc / madc: cw*1 + cw), and for madc > 0 every madc-th slot's
    add-with-carry is a multiply-add with carry (row*1 + x + carry), which
    ptxas issues as IMAD.X on the FMA pipe instead of IADD3.X on the ALU
    pipe; the carry flag chain is the same."""
    outs = [f'"+r"(row[{m}])' for m in range(TW)]
    idx_cw = idx_ncw = None
    if cin:
        idx_cw = len(outs)
        outs.append('"+r"(cw)')
    if cout:
        idx_ncw = len(outs)
        outs.append('"+r"(ncw)')
    ins = []
    e_idx = {}
    for m in range(TW):
        e_idx[m] = len(outs) + len(ins)
        ins.append(f'"r"(e[{m}])')
    one = len(outs) + len(ins)
    ins.append('"r"(one)')
    lines = ["{", ".reg .u32 x, t;"]
    if cin:
        lines.append(f"mad.lo.cc.u32 %{idx_cw}, %{idx_cw}, %{one}, %{idx_cw};")
    for m in range(TW):
        lines.append(f"and.b32 x, %{m}, %{e_idx[m]};")
        first = (m == 0 and not cin)
        last_no_out = (m == TW - 1 and not cout)
        cc = "" if last_no_out else ".cc"
        if madc and m % madc == madc - 1:
            op = "mad.lo" if first else "madc.lo"
            lines.append(f"{op}{cc}.u32 t, %{m}, %{one}, x;")
        else:
            op = "add" if first else "addc"
            lines.append(f"{op}{cc}.u32 t, %{m}, x;")
        lines.append(f"lop3.b32 %{m}, t, %{m}, x, 0xF6;")
    if cout:
        lines.append(f"madc.lo.u32 %{idx_ncw}, %{idx_ncw}, %{one}, %{idx_ncw};")
    lines.append("}")
    body = "\n".join(f'      "{ln}\\n\\t"' for ln in lines)
    sig = (f"template <>\n__device__ __forceinline__ void dp_tile_eqf<{TW}, {str(cin).lower()}, "
           f"{str(cout).lower()}, {madc}>(uint32_t (&row)[{TW}], const uint32_t (&e)[{TW}], uint32_t &cw, "
           f"uint32_t &ncw, uint32_t one) {{\n")
    unused = []
    if not cin:
        unused.append("cw")
    if not cout:
        unused.append("ncw")
    void = "".join(f"  (void){u};\n" for u in unused)
    return (sig + void + "  asm(\n" + body + "\n      : " + ", ".join(outs) + "\n      : " + ", ".join(ins) +
            ");\n}\n")


# dp_tile_eqf variants generated: madc = 0 only.  Every 2nd or 3rd slot's
# add as IMAD.X (madc = 2, 3) was swept on GB300 (1M DNA, s=0.85) and ran
# at 0.97x and 0.98x of madc = 0.
MADC = (0,)


def main() -> None:
    parts = ["// dp_asm.cuh — generated by gen_dp_asm.py; do not edit by hand.\n"
             "// One residue (column) update of a TW-slot register tile of the banded\n"
             "// bit-parallel LCS for P bit planes; see gen_dp_asm.py for the algebra.\n"
             "#pragma once\n#include <stdint.h>\n\nnamespace ngia {\n\n"
             "template <int P, int TW, bool CIN, bool COUT>\n"
             "__device__ __forceinline__ void dp_tile(uint32_t (&row)[TW], const uint32_t (&pl)[P][TW],\n"
             "                                        const uint32_t (&mk)[P], uint32_t &cw, uint32_t &ncw);\n\n"
             "template <int TW, bool CIN, bool COUT>\n"
             "__device__ __forceinline__ void dp_tile_eq(uint32_t (&row)[TW], const uint32_t (&e)[TW], uint32_t &cw,\n"
             "                                           uint32_t &ncw);\n\n"
             "template <int TW, bool CIN, bool COUT, int MADC>\n"
             "__device__ __forceinline__ void dp_tile_eqf(uint32_t (&row)[TW], const uint32_t (&e)[TW], uint32_t &cw,\n"
             "                                            uint32_t &ncw, uint32_t one);\n\n"]
    for P in PLANES:
        for TW in WIDTHS:
            for cin, cout in ((False, False), (True, True)):
                parts.append(one(P, TW, cin, cout))
                parts.append("\n")
    for TW in WIDTHS:
        for cin, cout in ((False, False), (True, True)):
            parts.append(one_eq(TW, cin, cout))
            parts.append("\n")
    for madc in MADC:
        for TW in WIDTHS:
            for cin, cout in ((False, False), (True, True)):
                parts.append(one_eqf(TW, cin, cout, madc))
                parts.append("\n")
    parts.append("}  // namespace ngia\n")
    (Path(__file__).resolve().parent / "dp_asm.cuh").write_text("".join(parts))


if __name__ == "__main__":
    main()
