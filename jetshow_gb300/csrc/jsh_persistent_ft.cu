// jsh_persistent_ft.cu -- the mixed path's transfer kernels and launch
// sequence built with the Faraday-thick mode of the IQUV pass compiled in
// (requests with JSH_FLAG_FARADAY_THICK).  Same source as jsh_persistent.cu;
// the default build leaves the mode out, so requests that do not ask for it
// run exactly the kernels they ran before.
#define JSH_FARADAY_THICK_BUILD 1
#include "jsh_persistent.cu"
