// Stand-in for FSL's utils/log.h (see options.h). TEST INFRASTRUCTURE.
#pragma once
namespace Utilities {
class Log {};
class LogSingleton {
 public:
  static Log& getInstance() { static Log l; return l; }
};
}  // namespace Utilities
