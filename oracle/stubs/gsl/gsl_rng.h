/* Empty stand-in: the reference includes this header but calls no gsl_* symbol. Test infrastructure only. */
