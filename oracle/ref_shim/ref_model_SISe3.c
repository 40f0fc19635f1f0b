/* Exposes the static rate functions of the reference's src/models/SISe3.c
 * (compiled unmodified) to ref_driver.c.  Oracle test infrastructure. */
#include "models/SISe3.c"
TRFun ref_SISe3_tr[] = { &SISe3_S_1_to_I_1, &SISe3_I_1_to_S_1, &SISe3_S_2_to_I_2,
                         &SISe3_I_2_to_S_2, &SISe3_S_3_to_I_3, &SISe3_I_3_to_S_3 };
PTSFun ref_SISe3_pts = &SISe3_post_time_step;
