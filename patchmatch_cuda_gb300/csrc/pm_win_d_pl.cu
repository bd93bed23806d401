// Window sides 27..45 of the window-templated kernels, exact-gather sampler, slanted planes per pixel.
#define PM_GROUP_FN launch_group_d_pl
#define PM_HW false
#define PM_WINDOW_LIST(X) X(27) X(29) X(31) X(33) X(35) X(37) X(39) X(41) X(43) X(45)
#define PM_PL true
#include "pm_windows.inc"
