"""Regenerate ``_catalog_peaks.py`` from a scopyon catalog directory.

    python -m scopyon_gb300._make_catalog_peaks <scopyon>/catalog

For every fluorophore CSV it records the emission peak (integer nm) and the
sum of the normalised emission spectrum on the default 300-1000 nm grid, the
two numbers the image-formation path takes from the catalog.
"""

import os
import sys

from ._catalog import fluorophore_spectra


def main(catalog_dir):
    rows = []
    fdir = os.path.join(catalog_dir, "fluorophore")
    for fname in sorted(os.listdir(fdir)):
        if not fname.endswith(".csv"):
            continue
        name = fname[:-4]
        try:
            wl, norm = fluorophore_spectra(name, catalog_dir)
        except Exception as exc:  # malformed entries are skipped, as listed
            print("skip %s: %s" % (name, exc), file=sys.stderr)
            continue
        rows.append("    %r: (%d, %r)," % (name, int(round(wl / 1e-9)), norm))
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_catalog_peaks.py")
    with open(out, "w") as f:
        f.write('"""Emission peak (nm) and normalised-emission sum per fluorophore.\n\n'
                'Generated by _make_catalog_peaks.py from the scopyon catalog.\n"""\n\n')
        f.write("PEAKS = {\n" + "\n".join(rows) + "\n}\n")
    print("wrote %d entries to %s" % (len(rows), out))


if __name__ == "__main__":
    main(sys.argv[1])
