// Minimal stand-in for boost::format, enough for the reference's log lines
// ("%+.15f" applied to one value).  Written for this project; Boost itself is
// not installed.  Only used when compiling the reference sources as an oracle.
#pragma once
#include <iomanip>
#include <ostream>
#include <sstream>
#include <string>

namespace boost {
class format {
 public:
  explicit format(const char* spec) : spec_(spec) {}
  template <class T>
  format& operator%(const T& value) {
    std::ostringstream os;
    // "%+.15f": explicit sign, fixed notation, 15 digits after the point.
    os << std::showpos << std::fixed << std::setprecision(15) << value;
    text_ += os.str();
    return *this;
  }
  friend std::ostream& operator<<(std::ostream& os, const format& f) { return os << f.text_; }

 private:
  std::string spec_;
  std::string text_;
};
}  // namespace boost
