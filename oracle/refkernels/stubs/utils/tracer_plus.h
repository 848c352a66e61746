// Stand-in for FSL's utils/tracer_plus.h (see options.h). TEST INFRASTRUCTURE.
#pragma once
