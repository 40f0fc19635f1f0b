/* Exposes the static rate and post-time-step functions of the reference's
 * src/models/SISe_sp.c (compiled unmodified) to ref_driver.c.  Oracle test
 * infrastructure. */
#include "models/SISe_sp.c"
TRFun ref_SISe_sp_tr[] = { &SISe_sp_S_to_I, &SISe_sp_I_to_S };
PTSFun ref_SISe_sp_pts = &SISe_sp_post_time_step;
