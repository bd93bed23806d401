// Window sides 3..11 of the window-templated kernels, exact-gather sampler, slanted planes per pixel.
#define PM_GROUP_FN launch_group_a_pl
#define PM_HW false
#define PM_WINDOW_LIST(X) X(3) X(5) X(7) X(9) X(11)
#define PM_PL true
#include "pm_windows.inc"
