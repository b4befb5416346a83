/* Stand-in for boost::iostreams::filtering_istream: reads a whole file and
 * drops '#'-to-end-of-line comments, which is what AFEPack's comment filter
 * does (src/Miscellaneous.cpp:24-61).  Oracle build only. */
#pragma once
#include <istream>
#include <sstream>
#include <fstream>
#include <string>
#include <cstdio>
#include <cassert>
#include <climits>
namespace boost { namespace iostreams {
const int WOULD_BLOCK = -2;
struct input_filter {};
struct file_source {
  std::string name;
  file_source(const char* n) : name(n) {}
  file_source(const std::string& n) : name(n) {}
};
struct filtering_istream : std::istream {
  std::stringbuf buf;
  filtering_istream() : std::istream(nullptr) { rdbuf(&buf); }
  template <class F> void push(const F&) {}
  void push(const file_source& f) {
    std::ifstream in(f.name);
    if (!in) { setstate(std::ios::failbit); return; }
    std::string line, text;
    while (std::getline(in, line)) {
      std::string::size_type p = line.find('#');
      if (p != std::string::npos) line.erase(p);
      text += line;
      text += '\n';
    }
    buf.str(text);
    clear();
  }
};
template <class S> int get(S&) { return EOF; }
}}
