/*
 * Minimal stand-in for <boost/program_options.hpp>, written for this project.
 *
 * Boost is not installed in the build image.  The reference's util/config.h
 * includes this header only for its two command-line parsers
 * (util/config.h:117-195, 228-329); the oracle build never calls them, but
 * they are inline functions, so the names they use must exist and type-check.
 * Nothing here parses anything.
 */
#ifndef GLINT_ORACLE_PO_STUB_HPP
#define GLINT_ORACLE_PO_STUB_HPP

#include <string>
#include <ostream>

namespace boost {
namespace program_options {

struct value_semantic {};

template <class T>
inline value_semantic *value(T *) { return nullptr; }

class options_description {
public:
    explicit options_description(const std::string & = std::string()) {}
    struct adder {
        adder &operator()(const char *, const char *) { return *this; }
        adder &operator()(const char *, value_semantic *, const char *) { return *this; }
    };
    adder add_options() { return adder(); }
};

inline std::ostream &operator<<(std::ostream &os, const options_description &) { return os; }

class variables_map {
public:
    std::size_t count(const std::string &) const { return 0; }
};

struct parsed_options {};

inline parsed_options parse_command_line(int, char **, const options_description &) { return parsed_options(); }
inline void store(const parsed_options &, variables_map &) {}
inline void notify(variables_map &) {}

} // namespace program_options
} // namespace boost

#endif
