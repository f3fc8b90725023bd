// Minimal stand-in for boost::timer (oracle build only).
#ifndef ORACLE_SHIM_BOOST_TIMER_HPP
#define ORACLE_SHIM_BOOST_TIMER_HPP
#include <ctime>
namespace boost {
class timer {
 public:
  timer() : t0_(std::clock()) {}
  void restart() { t0_ = std::clock(); }
  double elapsed() const { return double(std::clock() - t0_) / CLOCKS_PER_SEC; }
 private:
  std::clock_t t0_;
};
}  // namespace boost
#endif
