// Window sides 19..25 of the window-templated kernels, exact-gather sampler.
#define PM_GROUP_FN launch_group_c
#define PM_HW false
#define PM_WINDOW_LIST(X) X(19) X(21) X(23) X(25)
#define PM_PL false
#include "pm_windows.inc"
