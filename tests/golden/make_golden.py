"""Extracts the golden table rows used to pin the oracle's table generator.

Source: the reference's exported force table
``examples/use_ForceTableGen/EM_TB_WANGJUN_W-HE_2010.pair`` (written by
``Export_ForceTable``, MD_TypeDef_ForceTable.F90:1315-1459).  Table ID #1 is the
Ackland-Thetford W-W FS potential (FS_Ackland_WW.F90); its four columns are
r*V(r) [eV*A], -r*dV/dr [eV], RHO [eV^2] and -dRHO/dr [eV^2/A] on the grid
r_i = (i*CSIV)^2 with NTAB = 10000 and Rmax = 10 A.

Tables #2-#5 of the same export go to ``wangjun_pair_rows.txt``: #2 He-He
(ZBL_EXP6_HeHe.F90), #3 He-W and #4 W-He (ZBL_ABINTIO_He_W_930.F90), #5 W-W Derlet et al.
(FS_PM_WW.F90), four columns each, at the rows of table #1 plus the rows around every
piece boundary of those functions.

Run once in a container that has the reference mounted; the output files are committed.
"""
import os
import sys

# root of the reference tree: $MSMPSCU_REFERENCE, else where this container mounts it;
# the first command-line argument overrides the whole path
REF_ROOT = os.environ.get("MSMPSCU_REFERENCE", "/root/reference")
SRC = os.path.join(REF_ROOT, "examples/use_ForceTableGen/EM_TB_WANGJUN_W-HE_2010.pair")
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ackland_ww_pair_rows.txt")
OUT2 = os.path.join(os.path.dirname(os.path.abspath(__file__)), "wangjun_pair_rows.txt")
# piece boundaries (A) of tables #2-#5: He-He 1.0, 1.3; He-W 1.5778 ... 3.5, switch 4.3, 7.3;
# Derlet knots
EDGES = [1.0, 1.3, 1.57783601880074, 1.94810507446527, 2.10799896717072, 2.22277348041534,
         2.32289959788322, 3.05974050760269, 3.5, 4.3, 5.8, 7.3, 2.46699, 2.604045, 2.7411, 2.8528,
         3.009066666666667, 3.13602, 3.165333333333333, 3.3216, 3.41924, 3.70246, 3.98568, 4.2689]


def main():
    src = sys.argv[1] if len(sys.argv) > 1 else SRC
    rows = {}
    with open(src) as fh:
        for line in fh:
            parts = line.split()
            if not parts or not parts[0].isdigit():
                continue
            i = int(parts[0])
            rows[i] = parts[1:22]          # r, then four columns for each of tables #1-#5
    keep = sorted(set(list(range(1, 11)) + list(range(25, 10001, 25)) +
                      list(range(5270, 5290)) + list(range(6620, 6640)) + [9999, 10000]))
    with open(OUT, "w") as fh:
        fh.write("# rows of EM_TB_WANGJUN_W-HE_2010.pair, table #1 (W-W Ackland-Thetford)\n")
        fh.write("# NTAB=10000 RMAX_A=10.0\n")
        fh.write("# index r_A rV_eVA mrdVdr_eV rho_eV2 mdrhodr_eV2perA\n")
        for i in keep:
            fh.write("%d %s\n" % (i, " ".join(rows[i][:5])))
    print("wrote", OUT, len(keep), "rows")
    near = set()
    for r in EDGES:
        c = int(round(10000 * (r / 10.0) ** 0.5))
        near.update(range(max(1, c - 3), min(10000, c + 3) + 1))
    keep2 = sorted(set(keep) | near)
    with open(OUT2, "w") as fh:
        fh.write("# rows of EM_TB_WANGJUN_W-HE_2010.pair, tables #2 He-He, #3 He-W, #4 W-He, #5 W-W Derlet\n")
        fh.write("# NTAB=10000 RMAX_A=10.0; per table: rV_eVA mrdVdr_eV rho_eV2 mdrhodr_eV2perA\n")
        fh.write("# index r_A then 16 columns\n")
        for i in keep2:
            fh.write("%d %s %s\n" % (i, rows[i][0], " ".join(rows[i][5:21])))
    print("wrote", OUT2, len(keep2), "rows")


if __name__ == "__main__":
    main()
