// cudimot.h - bound and prior kinds shared by the host parser, the kernels
// and model plugins. Same names and values as CUDIMOT's cudimot.h:16-17, so
// plugins and modelpriors files that refer to them keep their meaning.
#ifndef CUDIMOT_H_INCLUDED
#define CUDIMOT_H_INCLUDED
enum bound { NOBOUNDS, BMIN, BMAX, BMINMAX };
enum prior { NOPRIOR, GAUSSPRIOR, GAMMAPRIOR, ARDPRIOR, SINPRIOR, CUSTOM };
#endif
