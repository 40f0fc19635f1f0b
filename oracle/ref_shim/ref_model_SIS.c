/* Exposes the static rate functions of the reference's src/models/SIS.c
 * (compiled unmodified) to ref_driver.c.  Oracle test infrastructure. */
#include "models/SIS.c"
TRFun ref_SIS_tr[] = { &SIS_S_to_I, &SIS_I_to_R };
PTSFun ref_SIS_pts = &SIS_post_time_step;
