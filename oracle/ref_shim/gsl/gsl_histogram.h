/* gsl/gsl_histogram.h — ORACLE test infrastructure: included by the
   reference's data_types.h:26; solver.c and utils.c call no GSL routine. */
