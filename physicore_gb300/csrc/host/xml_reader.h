// xml_reader.h -- a small XML reader for PhysiCell settings files: elements,
// attributes, character data, comments, CDATA sections, processing instructions
// and the five predefined entities plus numeric character references.  DTDs are
// skipped.  It replaces the pugixml DOM the reference reads settings with
// (reactions-diffusion/biofvm/src/config_reader.cpp), offering the few queries that
// reader makes: child by name, next sibling by name, child by attribute value,
// attribute text and element text, with pugixml's text-to-value conversions.
#pragma once

#include <memory>
#include <string>
#include <string_view>
#include <vector>

namespace physicore::xml {

struct node
{
	std::string name;
	std::vector<std::pair<std::string, std::string>> attributes;
	std::string text; // character data directly inside the element, concatenated
	std::vector<std::unique_ptr<node>> children;
	node* parent = nullptr;

	// First child element called `name`, or nullptr.
	const node* child(std::string_view child_name) const;
	// The next element after this one, within the parent, called `name`, or nullptr.
	const node* next_sibling(std::string_view sibling_name) const;
	// First child element called `child_name` whose attribute `attr` equals `value`.
	const node* find_child_by_attribute(std::string_view child_name, std::string_view attr,
										std::string_view value) const;
	// The attribute's value, or nullptr when absent.
	const std::string* attribute(std::string_view attr) const;
};

// pugixml's conversions: as_double is strtod of the text (0 when empty or not a
// number); as_bool is true when the first character is one of 1 t T y Y; as_uint
// parses a decimal (or 0x hexadecimal) integer, 0 when absent.
double as_double(const std::string* text);
bool as_bool(const std::string* text);
unsigned long long as_uint(const std::string* text);
inline double as_double(const std::string& text) { return as_double(&text); }
inline bool as_bool(const std::string& text) { return as_bool(&text); }

struct document
{
	node root; // holds the top-level element(s) as children

	// Parses `text`; on malformed input returns false and sets `error` to a
	// description with the line number.
	bool parse(std::string_view text, std::string& error);
	bool load_file(const std::string& path, std::string& error);

	const node* child(std::string_view name) const { return root.child(name); }
};

} // namespace physicore::xml
