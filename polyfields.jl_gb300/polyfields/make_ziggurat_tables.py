"""Regenerate polyfields/ziggurat_tables.npz: the layer tables of the 256-layer normal ziggurat
(G. Marsaglia and W. W. Tsang, J. Stat. Softw. 5(8), 2000) as Julia's `randn` uses them.  The
tables use right edge r = 3.6541528853610088 and a 51-bit abscissa scale, with the layer area v
computed exactly from r.  They are built in 50-digit arithmetic and rounded once:

  k[i]: acceptance thresholds (integers on the 2^51 scale)
  w[i]: layer widths / 2^51
  f[i]: exp(-x_i^2 / 2) at the layer edges

Needs mpmath (here only; the package reads the committed .npz).

Usage:  python polyfields.jl_gb300/polyfields/make_ziggurat_tables.py
"""
import os

import numpy as np

R = 3.6541528853610088


def tables():
    import mpmath as mp
    with mp.workdps(50):
        r = mp.mpf(R)
        v = r * mp.exp(-r * r / 2) + mp.sqrt(mp.pi / 2) * mp.erfc(r / mp.sqrt(2))
        scale = mp.mpf(2) ** 51
        k = np.zeros(256, dtype=np.uint64)
        w = np.zeros(256)
        f = np.zeros(256)
        edge = r
        bottom = v / mp.exp(-edge * edge / 2)   # the bottom layer's width, tail included
        k[0] = int(mp.floor(edge / bottom * scale))
        w[0] = float(bottom / scale)
        w[255] = float(edge / scale)
        f[0] = 1.0
        f[255] = float(mp.exp(-edge * edge / 2))
        for i in range(254, 0, -1):
            nxt = mp.sqrt(-2 * mp.log(v / edge + mp.exp(-edge * edge / 2)))
            k[i + 1] = int(mp.floor(nxt / edge * scale))
            w[i] = float(nxt / scale)
            f[i] = float(mp.exp(-nxt * nxt / 2))
            edge = nxt
    return k, w, f


def main() -> None:
    k, w, f = tables()
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ziggurat_tables.npz")
    np.savez(dst, k=k, w=w, f=f)
    print(f"wrote {dst}")


if __name__ == "__main__":
    main()
