/* Exposes the static rate functions of the reference's src/models/SIR.c
 * (compiled unmodified) to ref_driver.c.  Oracle test infrastructure. */
#include "models/SIR.c"
TRFun ref_SIR_tr[] = { &SIR_S_to_I, &SIR_I_to_R };
PTSFun ref_SIR_pts = &SIR_post_time_step;
