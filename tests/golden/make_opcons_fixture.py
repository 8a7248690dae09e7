"""Copies the reference's valence spectrum EXAMPLE/Si_valence/opcons (the header
and every STRIDE-th of its 2000 write_val rows, starting with the first) into
tests/golden/opcons_Si_valence_rows.txt, the fixture of the opcons writer /
optical-constant tests.  Run once in a checkout that has the reference next to
it:

    python tests/golden/make_opcons_fixture.py /path/to/OCEAN
"""
import os
import sys

STRIDE = 5


def main(ref_root: str) -> None:
    src = os.path.join(ref_root, "EXAMPLE", "Si_valence", "opcons")
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "opcons_Si_valence_rows.txt")
    with open(src) as f:
        lines = f.read().splitlines()
    keep = [lines[0]] + lines[1::STRIDE]
    with open(dst, "w") as f:
        f.write("\n".join(keep) + "\n")
    lines = keep
    print(f"{len(lines)} lines -> {dst}")


if __name__ == "__main__":
    main(sys.argv[1])
