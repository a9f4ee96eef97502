/* Stand-in for MATLAB's matrix.h, which the reference header includes for its MEX
 * host types.  The device code compiled from the reference uses none of them. */
