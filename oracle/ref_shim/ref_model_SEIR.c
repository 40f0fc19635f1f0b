/* Exposes the static rate functions of the reference's src/models/SEIR.c
 * (compiled unmodified) to ref_driver.c.  Oracle test infrastructure. */
#include "models/SEIR.c"
TRFun ref_SEIR_tr[] = { &SEIR_S_to_E, &SEIR_E_to_I, &SEIR_I_to_R };
PTSFun ref_SEIR_pts = &SEIR_post_time_step;
