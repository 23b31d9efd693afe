// qudrip_gpu_params.hpp -- the reference's parameter-file reader
// (find_param.hpp: param_finder, find_param, find_param_tvec, convert,
// delete_space) for drivers that read `name = value` files the way its
// programs do.  Host code only; it needs nothing from the library.
//
// param_finder(fname) reads the file once: white space (std::isspace in the
// classic locale) is removed from each line, lines starting with '#' or
// without '=' are skipped, and the first definition of a name wins.
// find_param(name, value, warning) converts the text to value's type (or
// throws the name when it is missing and warning is set; otherwise leaves
// value unchanged); find_param_tvec fills a vector from one value or from the
// file named after a leading "--" (one value per line, '#' lines skipped,
// complex lines "re im").  Conversions are the reference's: floating types by
// std::stod (std::stold when out of range), int and long by std::stoi,
// strings as they are, std::complex<double> by operator>>.
#pragma once

#include <algorithm>
#include <complex>
#include <fstream>
#include <locale>
#include <sstream>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

namespace qudrip_gpu {

inline std::string delete_space(std::string s) {
  s.erase(std::remove_if(s.begin(), s.end(), [](char c) { return std::isspace(c, std::locale::classic()); }),
          s.end());
  return s;
}

template <class T>
struct param_convert {
  static T from(const std::string& s) {
    try {
      return static_cast<T>(std::stod(s));
    } catch (std::out_of_range&) {
      return static_cast<T>(std::stold(s));
    }
  }
};
template <>
struct param_convert<int> {
  static int from(const std::string& s) { return std::stoi(s); }
};
template <>
struct param_convert<long> {
  static long from(const std::string& s) { return std::stoi(s); }
};
template <>
struct param_convert<std::string> {
  static std::string from(const std::string& s) { return s; }
};
template <>
struct param_convert<std::complex<double>> {
  static std::complex<double> from(const std::string& s) {
    std::stringstream iss(s);
    std::complex<double> v(0.0, 0.0);
    iss >> v;
    return v;
  }
};

template <class T>
T convert(const std::string& s) {
  return param_convert<T>::from(s);
}

class param_finder {
 public:
  explicit param_finder(const std::string& fname) {
    std::ifstream f(fname);
    std::string oline;
    while (std::getline(f, oline)) {
      const std::string line = delete_space(oline);
      const auto peq = line.find('=');
      if ((!line.empty() && line[0] == '#') || peq == std::string::npos) continue;
      params_.insert({line.substr(0, peq), line.substr(peq + 1)});
    }
  }

  template <class T>
  void find_param(const std::string& name, T& value, int warning = 0) const {
    auto it = params_.find(name);
    if (it == params_.end()) {
      if (warning) throw name;
      return;
    }
    value = convert<T>(it->second);
  }

  template <class T>
  void find_param_tvec(const std::string& name, std::vector<T>& value, int warning = 0) const {
    auto it = params_.find(name);
    if (it == params_.end()) {
      if (warning) throw name;
      return;
    }
    const std::string& text = it->second;
    if (text.substr(0, 2) == "--") {
      std::ifstream f(text.substr(2));
      std::string line;
      for (size_t t = 0; t < value.size(); ++t) {
        while (std::getline(f, line) && !line.empty() && line[0] == '#') {
        }
        value[t] = from_line<T>(line);
      }
    } else {
      const T v = convert<T>(text);
      std::fill(value.begin(), value.end(), v);
    }
  }

 private:
  template <class T>
  static T from_line(const std::string& line) {
    return convert<T>(line);
  }
  std::unordered_map<std::string, std::string> params_;
};

template <>
inline std::complex<double> param_finder::from_line<std::complex<double>>(const std::string& line) {
  std::stringstream iss(line);
  double re = 0.0, im = 0.0;
  iss >> re >> im;
  return std::complex<double>(re, im);
}

}  // namespace qudrip_gpu
