/* Empty stand-in for <hdf5_hl.h> (oracle build only). */
#include "hdf5.h"
