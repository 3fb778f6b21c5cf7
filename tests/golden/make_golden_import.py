"""Fixtures for the import of tables the reference exported (Import_ForceTable and
Register_Imported_ForceTable, MDLIB/sor/Common/MD_TypeDef_ForceTable.F90:1463-1855).

Sources in the reference tree, the reference's own Export_ForceTable output:
  examples/NIST_Potentials/Cu_EAM/Cu1.eam.fs.setfl.{pair,embd}
      the EAM tables it made from the NIST setfl file Cu1.eam.fs.setfl (one Cu table each);
      MD_ForceLib_Register.F90:405-420 runs every NIST potential from such a pair of files
  examples/use_ForceTableGen/EM_TB_WANGJUN_W-HE_2010.{pair,embd}
      the five FS tables of the W-He library (W-W Ackland, He-He, He-W, W-He, W-W Derlet)

Each file is stored byte for byte, xz-compressed, as tests/golden/ref_<name>.xz, so the
tests (and the GPU machine, which has no reference tree) can import exactly the rows the
reference wrote.  Run once in a container that has the reference mounted; the outputs are
committed.
"""
import lzma
import os
import sys

# root of the reference tree: $MSMPSCU_REFERENCE, else where this container mounts it
REF_ROOT = os.environ.get("MSMPSCU_REFERENCE", "/root/reference")
FILES = {
    "cu1_setfl": "examples/NIST_Potentials/Cu_EAM/Cu1.eam.fs.setfl",
    "wangjun_w_he": "examples/use_ForceTableGen/EM_TB_WANGJUN_W-HE_2010",
}
HERE = os.path.dirname(os.path.abspath(__file__))


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else REF_ROOT
    for name, rel in FILES.items():
        for ext in ("pair", "embd"):
            src = os.path.join(root, rel + "." + ext)
            data = open(src, "rb").read()
            out = os.path.join(HERE, "ref_%s.%s.xz" % (name, ext))
            with open(out, "wb") as fh:
                fh.write(lzma.compress(data, preset=9 | lzma.PRESET_EXTREME))
            print(out, len(data), os.path.getsize(out))


if __name__ == "__main__":
    main()
