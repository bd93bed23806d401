// Window sides 27..45 of the window-templated kernels, texture-filtering sampler.
#define PM_GROUP_FN launch_group_d_hw
#define PM_HW true
#define PM_WINDOW_LIST(X) X(27) X(29) X(31) X(33) X(35) X(37) X(39) X(41) X(43) X(45)
#define PM_PL false
#include "pm_windows.inc"
