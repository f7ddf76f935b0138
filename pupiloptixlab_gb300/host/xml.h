// xml.h -- a small XML reader for mitsuba3-style scene files.
//
// Replaces the reference's use of pugixml (resource/xml/parser.cpp:22-59):
// elements, attributes, comments, the <?xml?> prolog and CDATA-free text are
// supported, which is all the scene format uses.  Errors carry the line.
#pragma once

#include <memory>
#include <string>
#include <utility>
#include <vector>

namespace Pupil::xml {

struct Node {
    std::string name;
    std::vector<std::pair<std::string, std::string>> attrs;
    std::vector<std::unique_ptr<Node>> children;
    int line = 0;

    const std::string *attr(const std::string &key) const;
    std::string attr_or(const std::string &key, const std::string &fallback) const;
};

// Parses `text`; returns nullptr and fills `error` on malformed input.
std::unique_ptr<Node> Parse(const std::string &text, std::string &error);

}  // namespace Pupil::xml
