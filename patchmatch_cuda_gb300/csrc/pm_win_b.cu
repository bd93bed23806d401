// Window sides 13..17 of the window-templated kernels, exact-gather sampler.
#define PM_GROUP_FN launch_group_b
#define PM_HW false
#define PM_WINDOW_LIST(X) X(13) X(15) X(17)
#define PM_PL false
#include "pm_windows.inc"
