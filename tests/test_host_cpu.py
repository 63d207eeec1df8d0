"""Host decisions of the Python mirror (kvs_gb300/marching_cubes.py) that run
without a GPU, against the reference's outputs in the golden fixtures: the
object colour (ColorMap::at, ColorMap.cpp:1043-1054) and the default
transfer function's table."""
import numpy as np

from kvs_gb300.marching_cubes import TransferFunction

from .helpers import golden


def test_default_table_is_the_references():
    _, arr = golden()
    assert np.array_equal(TransferFunction().table, arr["colormap256"].reshape(256, 3))


def test_color_at_matches_reference():
    _, arr = golden()
    tf = TransferFunction(256, arr["colormap256"])
    tf.setRange(-1.0, 2.0)
    assert tf.hasRange()
    for v, want in zip(arr["color_at_values"], arr["color_at_rgb"]):
        assert np.array_equal(tf.color_at(float(v)), want), (v, tf.color_at(float(v)), want)


def test_range_rules():
    tf = TransferFunction()
    assert not tf.hasRange()
    tf.setRange(0.5, 0.5 + 1e-7)   # kvs::Math::Equal: closer than 1e-6 is no range
    assert not tf.hasRange()
    c = tf.copy()
    c.setRange(0.0, 1.0)
    assert c.hasRange() and not tf.hasRange()
