/* Exposes the static rate functions of the reference's src/models/SISe.c
 * (compiled unmodified) to ref_driver.c.  Oracle test infrastructure. */
#include "models/SISe.c"
TRFun ref_SISe_tr[] = { &SISe_S_to_I, &SISe_I_to_S };
PTSFun ref_SISe_pts = &SISe_post_time_step;
