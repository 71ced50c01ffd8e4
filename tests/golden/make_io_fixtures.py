"""Generates the I/O fixtures from the reference's own scripts (run in the
build container, where the reference tree is mounted; the outputs are
committed because the tree does not travel):

  ref_header.fil   a SIGPROC file written by the reference's
                   write_sigproc_header (scripts/make_noise_fil_with_frb.py:27-46)
                   followed by 16 spectra of 64 channels
  ref_dada_header.txt  a DADA header from get_dada_header
                   (scripts/convert_fil_to_dada.py:14-30)

Usage: python tests/golden/make_io_fixtures.py <reference tree>   (or set HELLA_REF)
"""
import importlib.util
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def _load(path: Path, name: str):
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    src = path.read_text()
    # import only the definitions: the scripts run their work under __main__
    exec(compile(src, str(path), "exec"), mod.__dict__)
    return mod


def main(ref: str):
    scripts = Path(ref) / "scripts"
    sys.path.insert(0, str(scripts))  # the converter imports its sibling script
    fil = _load(scripts / "make_noise_fil_with_frb.py", "ref_fil")
    hdr = dict(nbits=8, nchans=64, fch1=468.75, foff=-93.75 / 64, tsamp=1.048576e-3, tstart=60000.25,
               source_name="FAKE_FRB", rawdatafile="fixture.fil", ibeam=3, nbeams=8, telescope_id=7)
    data = (np.arange(16 * 64, dtype=np.int64) * 37 % 251).astype(np.uint8).reshape(16, 64)
    with open(HERE / "ref_header.fil", "wb") as fh:
        fil.write_sigproc_header(fh, hdr)
        fh.write(data.tobytes())
    dada = _load(scripts / "convert_fil_to_dada.py", "ref_dada")
    text = dada.get_dada_header(1 << 20, 1 << 16, 5, 16)
    (HERE / "ref_dada_header.txt").write_text(text)
    print("wrote", HERE / "ref_header.fil", HERE / "ref_dada_header.txt")


if __name__ == "__main__":
    import os

    tree = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("HELLA_REF")
    if not tree:
        raise SystemExit("usage: python make_io_fixtures.py <reference tree>  (or set HELLA_REF)")
    main(tree)
