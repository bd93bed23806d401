// Window sides 19..25 of the window-templated kernels, exact-gather sampler, slanted planes per pixel.
#define PM_GROUP_FN launch_group_c_pl
#define PM_HW false
#define PM_WINDOW_LIST(X) X(19) X(21) X(23) X(25)
#define PM_PL true
#include "pm_windows.inc"
