/* hdf5_hl.h — ORACLE test infrastructure: included by the reference's
   data_types.h:14; nothing from it is used by solver.c or utils.c. */
#include "hdf5.h"
