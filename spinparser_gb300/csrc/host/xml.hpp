// Minimal XML reader for SpinParser's task, lattice and model files.
//
// The reference reads these files with boost::property_tree::read_xml
// (src/TaskFileParser.cpp:24, src/LatticeModelFactory.cpp:115,253).  What the readers
// need from it is: several top-level elements per file (res/lattices.xml has one
// <unitcell> after another, no common root), attributes, the text of leaf elements,
// comments and the <?xml ...?> prolog.  This parser produces exactly that as a small DOM.
#pragma once
#include <string>
#include <vector>
#include <utility>

namespace spn {

struct XmlNode {
    std::string name;
    std::vector<std::pair<std::string, std::string>> attrs;
    std::vector<XmlNode> children;
    std::string text;  // character data directly inside this element (concatenated)

    const std::string *attr(const std::string &key) const;
    const XmlNode *child(const std::string &key) const;  // first child with that name
    int count(const std::string &key) const;
};

// Parses a document; the returned node is a synthetic root whose children are the
// top-level elements.  Throws spn::Error on malformed input.
XmlNode xml_parse_string(const std::string &doc);
XmlNode xml_parse_file(const std::string &path);

// Serialises an element tree (used to write the task file back with a new status).
std::string xml_serialize(const XmlNode &root);

}  // namespace spn
