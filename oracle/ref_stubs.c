/* Oracle link stubs.  The reference's hydro path never reaches these
 * symbols; they live in I/O, mesh-gravity, lightcone and neutrino units that
 * need HDF5/FFTW/GSL, which the oracle does not compile.  Each one aborts, so any
 * unexpected use fails loudly instead of returning garbage. */
#include <stdio.h>
#include <stdlib.h>

#define ORACLE_UNREACHABLE(name)                                    \
  void name(void) {                                                 \
    fprintf(stderr, "oracle: unexpected call to %s\n", #name);      \
    abort();                                                        \
  }

ORACLE_UNREACHABLE(do_line_of_sight)
ORACLE_UNREACHABLE(gather_neutrino_consts)
ORACLE_UNREACHABLE(git_branch)
ORACLE_UNREACHABLE(git_date)
ORACLE_UNREACHABLE(git_revision)
ORACLE_UNREACHABLE(gpart_neutrino_mass_weight)
ORACLE_UNREACHABLE(gravity_props_struct_dump)
ORACLE_UNREACHABLE(gravity_props_struct_restore)
ORACLE_UNREACHABLE(gravity_props_update)
ORACLE_UNREACHABLE(gravity_props_update_MAC_choice)
ORACLE_UNREACHABLE(lightcone_clean)
ORACLE_UNREACHABLE(lightcone_dump_completed_shells)
ORACLE_UNREACHABLE(lightcone_flush_map_updates)
ORACLE_UNREACHABLE(lightcone_flush_particle_buffers)
ORACLE_UNREACHABLE(lightcone_init)
ORACLE_UNREACHABLE(lightcone_memory_use)
ORACLE_UNREACHABLE(lightcone_prepare_for_step)
ORACLE_UNREACHABLE(lightcone_struct_dump)
ORACLE_UNREACHABLE(lightcone_struct_restore)
ORACLE_UNREACHABLE(lightcone_trigger_map_update)
ORACLE_UNREACHABLE(lightcone_write_index)
ORACLE_UNREACHABLE(los_struct_dump)
ORACLE_UNREACHABLE(los_struct_restore)
ORACLE_UNREACHABLE(neutrino_response_struct_dump)
ORACLE_UNREACHABLE(neutrino_response_struct_restore)
ORACLE_UNREACHABLE(neutrino_seed_to_direction)
ORACLE_UNREACHABLE(neutrino_seed_to_fermi_dirac)
ORACLE_UNREACHABLE(output_list_check_selection)
ORACLE_UNREACHABLE(output_list_clean)
ORACLE_UNREACHABLE(output_list_init)
ORACLE_UNREACHABLE(output_list_read_next_time)
ORACLE_UNREACHABLE(output_options_clean)
ORACLE_UNREACHABLE(output_options_struct_dump)
ORACLE_UNREACHABLE(output_options_struct_restore)
ORACLE_UNREACHABLE(package_version)
ORACLE_UNREACHABLE(pm_mesh_allocate)
ORACLE_UNREACHABLE(pm_mesh_compute_potential)
ORACLE_UNREACHABLE(pm_mesh_free)
ORACLE_UNREACHABLE(pm_mesh_struct_dump)
ORACLE_UNREACHABLE(pm_mesh_struct_restore)
