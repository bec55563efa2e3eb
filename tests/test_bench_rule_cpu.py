"""bench.py's copy of the scheduled driver's layout rule, against the layouts
the driver launched for the manifold batch on a 152-SM GB300 (launch list:
lane pairs while 16384 and 8896 trajectories are live, six lanes at 3160)."""
import bench


def test_sched_lanes_matches_driver_choices():
    slots = 4.5 * 152
    assert bench.sched_lanes(16384, slots) == 2
    assert bench.sched_lanes(8896, slots) == 2
    assert bench.sched_lanes(3160, slots) == 6
    assert bench.sched_lanes(65536, 3.0 * 152) == 1
    assert bench.sched_lanes(1, slots) == 6
