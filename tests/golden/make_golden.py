"""Extracts the golden table rows used to pin the oracle's table generator.

Source: the reference's exported force table
``examples/use_ForceTableGen/EM_TB_WANGJUN_W-HE_2010.pair`` (written by
``Export_ForceTable``, MD_TypeDef_ForceTable.F90:1315-1459).  Table ID #1 is the
Ackland-Thetford W-W FS potential (FS_Ackland_WW.F90); its four columns are
r*V(r) [eV*A], -r*dV/dr [eV], RHO [eV^2] and -dRHO/dr [eV^2/A] on the grid
r_i = (i*CSIV)^2 with NTAB = 10000 and Rmax = 10 A.

Run once in a container that has the reference mounted; the output file is committed.
"""
import os
import sys

SRC = "/root/reference/examples/use_ForceTableGen/EM_TB_WANGJUN_W-HE_2010.pair"
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ackland_ww_pair_rows.txt")


def main():
    src = sys.argv[1] if len(sys.argv) > 1 else SRC
    rows = {}
    with open(src) as fh:
        for line in fh:
            parts = line.split()
            if not parts or not parts[0].isdigit():
                continue
            i = int(parts[0])
            rows[i] = parts[1:6]           # r, then table #1's four columns
    keep = sorted(set(list(range(1, 11)) + list(range(25, 10001, 25)) +
                      list(range(5270, 5290)) + list(range(6620, 6640)) + [9999, 10000]))
    with open(OUT, "w") as fh:
        fh.write("# rows of EM_TB_WANGJUN_W-HE_2010.pair, table #1 (W-W Ackland-Thetford)\n")
        fh.write("# NTAB=10000 RMAX_A=10.0\n")
        fh.write("# index r_A rV_eVA mrdVdr_eV rho_eV2 mdrhodr_eV2perA\n")
        for i in keep:
            fh.write("%d %s\n" % (i, " ".join(rows[i])))
    print("wrote", OUT, len(keep), "rows")


if __name__ == "__main__":
    main()
