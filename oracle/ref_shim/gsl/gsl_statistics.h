/* gsl/gsl_statistics.h — ORACLE test infrastructure: included by the
   reference's data_types.h:27; solver.c and utils.c call no GSL routine. */
