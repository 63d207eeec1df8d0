"""Write default_colormap.py: the reference's default colour table.

kvs::TransferFunction(256) builds its colour map with ColorMap::BrewerRdBu
(Source/Core/Visualization/Mapper/ColorMap.cpp:23,255-277), interpolated in
Lab space.  The mapper only needs the finished 256 x RGB table (colour is one
host-side lookup per call, MarchingCubes.cpp:239), so the table is taken from
the reference built under oracle/_ref and committed as data.

    python kvs_gb300/gen_default_colormap.py
"""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from oracle import ref  # noqa: E402  (generator only; the package never imports oracle)


def main():
    t = ref.default_colormap(256)
    lines = ['"""Default colour table of kvs::TransferFunction(256): ColorMap::BrewerRdBu',
             '(Source/Core/Visualization/Mapper/ColorMap.cpp:255-277), 256 x RGB.',
             'Generated by gen_default_colormap.py from the reference build."""',
             "", "BREWER_RDBU_256 = bytes(["]
    flat = t.reshape(-1).tolist()
    for i in range(0, len(flat), 24):
        lines.append("    " + ", ".join(str(v) for v in flat[i:i + 24]) + ",")
    lines.append("])")
    with open(os.path.join(HERE, "default_colormap.py"), "w") as f:
        f.write("\n".join(lines) + "\n")


if __name__ == "__main__":
    main()
