/* Exposes the static rate and post-time-step functions of the reference's
 * src/models/SISe3_sp.c (compiled unmodified) to ref_driver.c, in
 * SISe3_sp_run's transition order.  Oracle test infrastructure. */
#include "models/SISe3_sp.c"
TRFun ref_SISe3_sp_tr[] = { &SISe3_sp_S_1_to_I_1, &SISe3_sp_I_1_to_S_1,
                            &SISe3_sp_S_2_to_I_2, &SISe3_sp_I_2_to_S_2,
                            &SISe3_sp_S_3_to_I_3, &SISe3_sp_I_3_to_S_3 };
PTSFun ref_SISe3_sp_pts = &SISe3_sp_post_time_step;
