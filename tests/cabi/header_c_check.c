/* The public header must compile as C (no C++ in the ABI): every declaration
 * is taken by address so a signature change shows up as a type error here. */
#include "gansu_gb300.h"

int (*p_create)(const hf_primitive_shell*, int, const double*, int, const hf_atom*, int, double, hf_engine**) =
    hf_engine_create;
int (*p_rhf)(hf_engine*, int, const hf_scf_options*, hf_scf_result*, double*, double*, double*, double*) =
    hf_rhf_scf;
int (*p_noalloc)(const double*, const double*, double*, int, int, void*) = hf_compute_fock_diis_noalloc;
void (*p_defaults)(hf_scf_options*) = hf_scf_options_default;
const char* (*p_err)(void) = hf_last_error;
