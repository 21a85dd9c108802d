"""Host mirror of the template build: the star list and the stamp window sizes that
define the build's work unit (bin updates)."""
import numpy as np


def test_stamp_window_sizes():
    from sfhgpu.templates import stamp_bin_updates
    xe = np.linspace(0.0, 1.0, 101)   # 100 colour bins of 0.01
    ye = np.linspace(0.0, 2.0, 101)   # 100 magnitude bins of 0.02
    e = (xe, ye)
    # a star in the middle, sigma = 0.3 pixel in x and 1.25 pixel in y
    x, y, sx, sy = 0.5, 1.0, 0.003, 0.025
    # GaussianPSFAsymmetric: size (ceil 3, ceil 12.5) = (3, 13), offsets (1, 6): 3 x 13
    assert stamp_bin_updates([x], [y], [sx], [sy], 0, e)[0] == 3 * 13
    # GaussianPSFCovariant: half widths round(15*0.3/2) = 2, round(10*1.25/2) = 6: 5 x 13
    assert stamp_bin_updates([x], [y], [sx], [sy], 1, e)[0] == 5 * 13
    assert stamp_bin_updates([x], [y], [sx], [sy], -1, e)[0] == 5 * 13
    # clipped at the first colour bin: centre pixel 1, window [1, 3] -> 3 wide
    assert stamp_bin_updates([0.004], [y], [sx], [sy], 1, e)[0] == 3 * 13
    # a corner star whose clipped window is one bin wide adds nothing (:359, :401)
    assert stamp_bin_updates([-0.0051], [y], [1e-6], [sy], 0, e)[0] == 0
    # a very wide star covers the whole grid
    assert stamp_bin_updates([x], [y], [5.0], [5.0], 1, e)[0] == 100 * 100


def test_star_list_feeds_the_device_template(sfh):
    """partial_cmd_smooth_stars + bin_cmd_smooth is partial_cmd_smooth."""
    from sfhgpu import synthetic as S
    from sfhgpu.templates import partial_cmd_smooth_stars
    w = S.small()
    m, mags = S.isochrone(8.5, -1.0, 120)
    x, y, sx, sy, wt, cov, e = partial_cmd_smooth_stars(
        m, list(mags), S.error_funcs(), 1, (0, 1), S.imf(), S.completeness_funcs(), dmod=25.0,
        edges=(w.xedges, w.yedges))
    assert cov == 1 and x.size == y.size == sx.size == sy.size == wt.size > 10
    assert np.all(np.diff(e[0]) > 0) and np.all(wt >= 0)
