// Window sides 13..17 of the window-templated kernels, texture-filtering sampler, slanted planes per pixel.
#define PM_GROUP_FN launch_group_b_hw_pl
#define PM_HW true
#define PM_WINDOW_LIST(X) X(13) X(15) X(17)
#define PM_PL true
#include "pm_windows.inc"
