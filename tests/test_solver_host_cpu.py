"""Host-side pieces of the simulator module that need no GPU."""
import numpy as np

from reduced_mpm_stress_training_gb300.solver import MPM_Simulator_WARP, flatten2nD


def test_flatten2nD_is_the_c_order_multi_index():
    """engine_stress/mpm_solver_warp.py:14-22."""
    for shape in [(4, 5, 6), (7,), (3, 3, 3, 3)]:
        for i in range(int(np.prod(shape))):
            assert flatten2nD(i, shape) == [int(j) for j in np.unravel_index(i, shape)]
    assert flatten2nD(130, (4, 5, 6)) == [4, 1, 4]   # the first index is not bounded, as there


def test_simulator_has_every_method_of_the_reference():
    names = ["initialize", "set_parameters", "load_from_sampling", "p2g2p", "experiment_for_C", "p2g2p_reduced",
             "load_x_initial_from_tensor", "load_mass_from_tensor", "load_uvF_from_tensor", "load_C_from_tensor",
             "load_uvstress_from_tensor", "load_uvFstress_from_h5", "export_uvFstress_from_warp",
             "particle_position2obj", "particle_F_norm2obj", "save_data_at_frame", "add_surface_collider",
             "add_surface_collider2", "add_bounding_box", "set_velocity_on_infinite_plane",
             "set_column_moving_as_circle", "set_rotation_on_disk", "set_velocity_on_cube", "add_sphere_leader"]
    missing = [n for n in names if not callable(getattr(MPM_Simulator_WARP, n, None))]
    assert not missing, missing
