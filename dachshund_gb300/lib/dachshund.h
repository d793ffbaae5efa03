// Umbrella header with the reference's name (lib/dachshund.h).
#ifndef DS_GB300_CXX_DACHSHUND_H
#define DS_GB300_CXX_DACHSHUND_H

#include "linalg.h"
#include "map.h"
#include "map_covar.h"
#include "pcg.h"
#include "pixel.h"
#include "signal_covar.h"
#include "timer.h"
#include "util.h"
#include "wf_vector.h"

#endif
