// Window sides 3..11 of the window-templated kernels, exact-gather sampler.
#define PM_GROUP_FN launch_group_a
#define PM_HW false
#define PM_WINDOW_LIST(X) X(3) X(5) X(7) X(9) X(11)
#define PM_PL false
#include "pm_windows.inc"
