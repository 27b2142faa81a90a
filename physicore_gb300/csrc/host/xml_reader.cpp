// xml_reader.cpp -- see xml_reader.h.  A recursive-descent reader over the whole
// file held in memory; element nesting is tracked with an explicit stack.
#include "xml_reader.h"

#include <cctype>
#include <cstdlib>
#include <fstream>
#include <sstream>

namespace physicore::xml {

const node* node::child(std::string_view child_name) const
{
	for (const auto& c : children)
		if (c->name == child_name)
			return c.get();
	return nullptr;
}

const node* node::next_sibling(std::string_view sibling_name) const
{
	if (!parent)
		return nullptr;
	bool after = false;
	for (const auto& c : parent->children)
	{
		if (after && c->name == sibling_name)
			return c.get();
		if (c.get() == this)
			after = true;
	}
	return nullptr;
}

const node* node::find_child_by_attribute(std::string_view child_name, std::string_view attr,
										  std::string_view value) const
{
	for (const auto& c : children)
		if (c->name == child_name)
			if (const std::string* v = c->attribute(attr); v && *v == value)
				return c.get();
	return nullptr;
}

const std::string* node::attribute(std::string_view attr) const
{
	for (const auto& a : attributes)
		if (a.first == attr)
			return &a.second;
	return nullptr;
}

double as_double(const std::string* text)
{
	if (!text || text->empty())
		return 0.0;
	return std::strtod(text->c_str(), nullptr);
}

bool as_bool(const std::string* text)
{
	if (!text)
		return false;
	std::size_t i = 0;
	while (i < text->size() && std::isspace(static_cast<unsigned char>((*text)[i])))
		i++;
	if (i == text->size())
		return false;
	const char c = (*text)[i];
	return c == '1' || c == 't' || c == 'T' || c == 'y' || c == 'Y';
}

unsigned long long as_uint(const std::string* text)
{
	if (!text || text->empty())
		return 0;
	return std::strtoull(text->c_str(), nullptr, 0);
}

namespace {

struct reader
{
	std::string_view s;
	std::size_t i = 0;
	std::string error;

	bool fail(const std::string& what)
	{
		std::size_t line = 1;
		for (std::size_t k = 0; k < i && k < s.size(); k++)
			line += s[k] == '\n';
		error = what + " at line " + std::to_string(line);
		return false;
	}

	bool starts(std::string_view p) const { return s.substr(i, p.size()) == p; }

	static bool name_char(char c)
	{
		return std::isalnum(static_cast<unsigned char>(c)) || c == '_' || c == '-' || c == '.' || c == ':' ||
			   static_cast<unsigned char>(c) >= 0x80;
	}

	void skip_space()
	{
		while (i < s.size() && std::isspace(static_cast<unsigned char>(s[i])))
			i++;
	}

	bool read_name(std::string& out)
	{
		const std::size_t b = i;
		while (i < s.size() && name_char(s[i]))
			i++;
		if (i == b)
			return fail("expected a name");
		out.assign(s.substr(b, i - b));
		return true;
	}

	// Skips up to and including `end`.
	bool skip_past(std::string_view end, const char* what)
	{
		const std::size_t k = s.find(end, i);
		if (k == std::string_view::npos)
			return fail(std::string("unterminated ") + what);
		i = k + end.size();
		return true;
	}

	static void put_utf8(std::string& out, unsigned long cp)
	{
		if (cp < 0x80)
			out += static_cast<char>(cp);
		else if (cp < 0x800)
		{
			out += static_cast<char>(0xC0 | (cp >> 6));
			out += static_cast<char>(0x80 | (cp & 0x3F));
		}
		else if (cp < 0x10000)
		{
			out += static_cast<char>(0xE0 | (cp >> 12));
			out += static_cast<char>(0x80 | ((cp >> 6) & 0x3F));
			out += static_cast<char>(0x80 | (cp & 0x3F));
		}
		else
		{
			out += static_cast<char>(0xF0 | (cp >> 18));
			out += static_cast<char>(0x80 | ((cp >> 12) & 0x3F));
			out += static_cast<char>(0x80 | ((cp >> 6) & 0x3F));
			out += static_cast<char>(0x80 | (cp & 0x3F));
		}
	}

	// Appends s[b, e) to out with entity and character references decoded.
	bool decode(std::size_t b, std::size_t e, std::string& out)
	{
		for (std::size_t k = b; k < e; k++)
		{
			if (s[k] != '&')
			{
				out += s[k];
				continue;
			}
			const std::size_t semi = s.find(';', k);
			if (semi == std::string_view::npos || semi >= e)
			{
				i = k;
				return fail("unterminated entity reference");
			}
			const std::string_view ent = s.substr(k + 1, semi - k - 1);
			if (ent == "lt")
				out += '<';
			else if (ent == "gt")
				out += '>';
			else if (ent == "amp")
				out += '&';
			else if (ent == "quot")
				out += '"';
			else if (ent == "apos")
				out += '\'';
			else if (!ent.empty() && ent[0] == '#')
			{
				const bool hex = ent.size() > 1 && (ent[1] == 'x' || ent[1] == 'X');
				const std::string digits(ent.substr(hex ? 2 : 1));
				char* end = nullptr;
				const unsigned long cp = std::strtoul(digits.c_str(), &end, hex ? 16 : 10);
				if (digits.empty() || *end != '\0' || cp > 0x10FFFF)
				{
					i = k;
					return fail("bad character reference");
				}
				put_utf8(out, cp);
			}
			else
			{
				i = k;
				return fail("unknown entity &" + std::string(ent) + ";");
			}
			k = semi;
		}
		return true;
	}

	bool read_attributes(node& n, bool& self_closing)
	{
		self_closing = false;
		for (;;)
		{
			skip_space();
			if (i >= s.size())
				return fail("unterminated start tag <" + n.name + ">");
			if (s[i] == '>')
			{
				i++;
				return true;
			}
			if (starts("/>"))
			{
				i += 2;
				self_closing = true;
				return true;
			}
			std::string key;
			if (!read_name(key))
				return false;
			skip_space();
			if (i >= s.size() || s[i] != '=')
				return fail("expected '=' after attribute " + key);
			i++;
			skip_space();
			if (i >= s.size() || (s[i] != '"' && s[i] != '\''))
				return fail("expected a quoted value for attribute " + key);
			const char q = s[i++];
			const std::size_t e = s.find(q, i);
			if (e == std::string_view::npos)
				return fail("unterminated value of attribute " + key);
			std::string value;
			if (!decode(i, e, value))
				return false;
			i = e + 1;
			n.attributes.emplace_back(std::move(key), std::move(value));
		}
	}

	bool parse(node& root)
	{
		std::vector<node*> open { &root };
		while (i < s.size())
		{
			node& cur = *open.back();
			if (s[i] != '<')
			{
				const std::size_t e = std::min(s.find('<', i), s.size());
				if (open.size() == 1)
				{
					for (std::size_t k = i; k < e; k++)
						if (!std::isspace(static_cast<unsigned char>(s[k])))
							return fail("character data outside the root element");
				}
				else if (!decode(i, e, cur.text))
					return false;
				i = e;
				continue;
			}
			if (starts("<!--"))
			{
				if (!skip_past("-->", "comment"))
					return false;
			}
			else if (starts("<![CDATA["))
			{
				const std::size_t b = i + 9;
				i = b;
				if (!skip_past("]]>", "CDATA section"))
					return false;
				if (open.size() == 1)
					return fail("CDATA outside the root element");
				cur.text.append(s.substr(b, i - 3 - b));
			}
			else if (starts("<?"))
			{
				if (!skip_past("?>", "processing instruction"))
					return false;
			}
			else if (starts("<!"))
			{
				// DOCTYPE, possibly with an internal subset in brackets
				int depth = 0;
				for (; i < s.size(); i++)
				{
					if (s[i] == '[')
						depth++;
					else if (s[i] == ']')
						depth--;
					else if (s[i] == '>' && depth <= 0)
						break;
				}
				if (i >= s.size())
					return fail("unterminated declaration");
				i++;
			}
			else if (starts("</"))
			{
				i += 2;
				std::string name;
				if (!read_name(name))
					return false;
				skip_space();
				if (i >= s.size() || s[i] != '>')
					return fail("malformed end tag </" + name);
				i++;
				if (open.size() == 1 || name != cur.name)
					return fail("end tag </" + name + "> does not match <" + (open.size() == 1 ? "" : cur.name) + ">");
				open.pop_back();
			}
			else
			{
				i++;
				auto n = std::make_unique<node>();
				if (!read_name(n->name))
					return false;
				bool self_closing;
				if (!read_attributes(*n, self_closing))
					return false;
				if (open.size() == 1 && !root.children.empty())
					return fail("more than one root element");
				n->parent = &cur;
				node* raw = n.get();
				cur.children.push_back(std::move(n));
				if (!self_closing)
					open.push_back(raw);
			}
		}
		if (open.size() != 1)
			return fail("unterminated element <" + open.back()->name + ">");
		if (root.children.empty())
			return fail("no root element");
		return true;
	}
};

} // namespace

bool document::parse(std::string_view text, std::string& error)
{
	root = node {};
	reader r;
	r.s = text;
	if (!r.parse(root))
	{
		error = r.error;
		root = node {};
		return false;
	}
	return true;
}

bool document::load_file(const std::string& path, std::string& error)
{
	std::ifstream f(path, std::ios::binary);
	if (!f)
	{
		error = "cannot open file";
		return false;
	}
	std::ostringstream ss;
	ss << f.rdbuf();
	return parse(ss.str(), error);
}

} // namespace physicore::xml
