// InputParser.hpp -- the command-line reader of TBSLA's driver programs
// (src/cpp/include/tbsla/cpp/utils/InputParser.hpp; its behaviour:
// src/cpp/utils/InputParser.cpp:4-21).  Same class and members, so that the
// reference's apps build against the drop-in unchanged.
#ifndef TBSLA_DROPIN_INPUTPARSER_HPP
#define TBSLA_DROPIN_INPUTPARSER_HPP

#include <string>
#include <vector>

class InputParser {
  public:
    // keeps argv[1 .. argc-1]
    InputParser(int &argc, char **argv);
    // the argument after the first occurrence of `option`, or default_opt
    // when the option is absent or last
    std::string get_opt(const std::string &option, const std::string default_opt = std::string("")) const;
    // whether `option` occurs among the arguments
    bool has_opt(const std::string &option) const;
  private:
    std::vector<std::string> params;
};

#endif
