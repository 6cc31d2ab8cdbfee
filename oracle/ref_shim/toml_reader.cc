// Project-written TOML-subset reader implementing the reference's reader API
// (src/reader.hh:9-53) in place of src/reader.cc, whose toml11 dependency is
// an empty git submodule in the reference checkout.
//
// Test infrastructure only: it lets the reference be compiled as the oracle.
// Supported TOML: comments, bare/quoted keys, basic and literal strings,
// integers, floats, booleans, (multi-line) arrays, inline tables, [table]
// headers and `baseinputfile` merging as in the reference (src/reader.cc:202-220).
// That is the subset every examples/*.toml of the reference uses.

#include "reader.hh"

#include <cstdlib>
#include <fstream>
#include <iostream>
#include <map>
#include <sstream>
#include <stdexcept>

#include "utils.hh"

class Node {
public:
	enum Kind { TABLE, ARRAY, STRING, INT, FLOAT, BOOL };
	Kind kind = TABLE;
	std::string s;
	long long i = 0;
	double f = 0;
	bool b = false;
	std::vector<std::shared_ptr<Node>> arr;
	std::vector<std::pair<std::string, std::shared_ptr<Node>>> tab;

	const Node *find(const std::string &k) const {
		if (kind != TABLE) return nullptr;
		for (const auto &p : tab) if (p.first == k) return p.second.get();
		return nullptr;
	}
	Node *find_mut(const std::string &k) {
		for (auto &p : tab) if (p.first == k) return p.second.get();
		return nullptr;
	}
};

namespace {

struct Parser {
	std::string src;
	size_t pos = 0;
	std::string file;

	[[noreturn]] void fail(const std::string &m) {
		size_t line = 1; for (size_t k = 0; k < pos && k < src.size(); k++) if (src[k] == '\n') line++;
		std::ostringstream o; o << file << ":" << line << ": " << m;
		throw std::runtime_error(o.str());
	}
	bool eof() const { return pos >= src.size(); }
	char peek() const { return eof() ? '\0' : src[pos]; }

	void skip_ws_line() {            // spaces/tabs and comments, not newlines
		while (!eof()) {
			char c = src[pos];
			if (c == ' ' || c == '\t' || c == '\r') pos++;
			else if (c == '#') { while (!eof() && src[pos] != '\n') pos++; }
			else break;
		}
	}
	void skip_ws_all() {             // including newlines
		while (!eof()) {
			skip_ws_line();
			if (!eof() && src[pos] == '\n') pos++; else break;
		}
	}

	std::string parse_key() {
		skip_ws_line();
		char c = peek();
		if (c == '"' || c == '\'') return parse_string();
		size_t st = pos;
		while (!eof()) {
			c = src[pos];
			if (isalnum((unsigned char)c) || c == '_' || c == '-') pos++; else break;
		}
		if (pos == st) fail("expected a key");
		return src.substr(st, pos - st);
	}

	std::string parse_string() {
		char q = src[pos];
		if (src.compare(pos, 3, std::string(3, q)) == 0) fail("multi-line strings are not supported");
		pos++;
		std::string out;
		while (true) {
			if (eof() || src[pos] == '\n') fail("unterminated string");
			char c = src[pos++];
			if (c == q) break;
			if (c == '\\' && q == '"') {
				if (eof()) fail("bad escape");
				char e = src[pos++];
				switch (e) {
					case 'n': out += '\n'; break;
					case 't': out += '\t'; break;
					case '"': out += '"'; break;
					case '\\': out += '\\'; break;
					default: out += '\\'; out += e; break;
				}
			} else out += c;
		}
		return out;
	}

	std::shared_ptr<Node> parse_value() {
		skip_ws_line();
		auto n = std::make_shared<Node>();
		char c = peek();
		if (c == '"' || c == '\'') { n->kind = Node::STRING; n->s = parse_string(); return n; }
		if (c == '[') {
			pos++; n->kind = Node::ARRAY;
			while (true) {
				skip_ws_all();
				if (peek() == ']') { pos++; break; }
				n->arr.push_back(parse_value());
				skip_ws_all();
				if (peek() == ',') { pos++; continue; }
				if (peek() == ']') { pos++; break; }
				fail("expected ',' or ']' in array");
			}
			return n;
		}
		if (c == '{') {
			pos++; n->kind = Node::TABLE;
			skip_ws_line();
			if (peek() == '}') { pos++; return n; }
			while (true) {
				std::string k = parse_key();
				skip_ws_line();
				if (peek() != '=') fail("expected '=' in inline table");
				pos++;
				n->tab.emplace_back(k, parse_value());
				skip_ws_line();
				if (peek() == ',') { pos++; continue; }
				if (peek() == '}') { pos++; break; }
				fail("expected ',' or '}' in inline table");
			}
			return n;
		}
		size_t st = pos;
		while (!eof()) {
			c = src[pos];
			if (c == ',' || c == ']' || c == '}' || c == '\n' || c == '#' || c == ' ' || c == '\t' || c == '\r') break;
			pos++;
		}
		std::string tok = src.substr(st, pos - st);
		if (tok == "true" || tok == "false") { n->kind = Node::BOOL; n->b = tok == "true"; return n; }
		std::string clean; for (char ch : tok) if (ch != '_') clean += ch;
		if (clean.empty()) fail("expected a value");
		bool isfloat = clean.find_first_of(".eE") != std::string::npos || clean == "inf" || clean == "nan";
		char *end = nullptr;
		if (isfloat) {
			n->kind = Node::FLOAT; n->f = strtod(clean.c_str(), &end);
		} else {
			n->kind = Node::INT; n->i = strtoll(clean.c_str(), &end, 0);
		}
		if (end == nullptr || *end != '\0') fail("cannot parse value '" + tok + "'");
		return n;
	}

	Node parse_document() {
		Node root; root.kind = Node::TABLE;
		Node *cur = &root;
		while (true) {
			skip_ws_all();
			if (eof()) break;
			if (peek() == '[') {
				pos++;
				if (peek() == '[') fail("arrays of tables are not supported");
				Node *t = &root;
				while (true) {
					std::string k = parse_key();
					Node *nx = t->find_mut(k);
					if (nx == nullptr) {
						auto nn = std::make_shared<Node>(); nn->kind = Node::TABLE;
						t->tab.emplace_back(k, nn); nx = nn.get();
					}
					t = nx;
					skip_ws_line();
					if (peek() == '.') { pos++; continue; }
					if (peek() == ']') { pos++; break; }
					fail("bad table header");
				}
				cur = t;
				continue;
			}
			std::string k = parse_key();
			skip_ws_line();
			if (peek() != '=') fail("expected '=' after key '" + k + "'");
			pos++;
			auto v = parse_value();
			if (cur->find(k) != nullptr) fail("duplicate key '" + k + "'");
			cur->tab.emplace_back(k, v);
			skip_ws_line();
			if (!eof() && peek() != '\n') fail("trailing characters after value of '" + k + "'");
		}
		return root;
	}
};

Node parse_toml_file(const std::string &fname)
{
	std::ifstream in(fname, std::ios::binary);
	if (!in) throw std::runtime_error("cannot open '" + fname + "'");
	std::stringstream ss; ss << in.rdbuf();
	Parser p; p.src = ss.str(); p.file = fname;
	return p.parse_document();
}

const Node &child(const Node &n, const std::string &name)
{
	const Node *c = n.find(name);
	if (c == nullptr) throw std::runtime_error("key '" + name + "' not found");
	return *c;
}

double as_number(const Node &v)
{
	if (v.kind == Node::FLOAT) return v.f;
	if (v.kind == Node::INT) return (double)v.i;
	throw std::runtime_error("value is not a number");
}

}  // namespace

InputNode::InputNode(const Node n, const std::string &label, const InputNode *parent)
	: n_(std::make_shared<Node>(n)), label_(label), parent_(parent) {}

size_t InputNode::size() const
{
	const Node &v = n();
	if (v.kind == Node::ARRAY) return v.arr.size();
	if (v.kind == Node::TABLE) return v.tab.size();
	if (v.kind == Node::STRING) return v.s.size();
	throw std::runtime_error("size() of a scalar value");
}

const Node &InputNode::n() const { return *n_; }

bool InputNode::contains(const std::string &name) const
{
	return n().find(name) != nullptr;
}

InputNode InputNode::operator[](unsigned int index) const
{
	const Node &v = n();
	if (v.kind != Node::ARRAY || index >= v.arr.size()) throw std::runtime_error("array index out of range");
	std::ostringstream oss; oss << '[' << index << ']';
	return InputNode(*v.arr[index], oss.str(), this);
}

InputNode InputNode::operator[](const std::string &s) const
{
	return InputNode(child(n(), s), s, this);
}

void InputNode::set_used()
{
	for (const auto &p : n().tab) {
		UsedTomlKey use; use.name = p.first; use.used = false;
		used.push_back(use);
	}
}

void InputNode::add_used(const string &name)
{
	auto i = 0u; while (i < used.size() && used[i].name != name) i++;
	if (i < used.size()) used[i].used = true;
}

void InputNode::check_used(string name)
{
	vector<string> not_used;
	for (const auto &use : used) if (use.used == false) not_used.push_back(use.name);
	if (not_used.size() > 0) {
		cout << "WARNING! In '" << name << "' unused quantities:";
		for (const auto &u : not_used) cout << " '" << u << "'";
		cout << endl << endl;
	}
}

std::string InputNode::stringfield_unchecked(const std::string &name)
{
	add_used(name);
	const Node &v = child(n(), name);
	if (v.kind != Node::STRING) throw std::runtime_error("'" + name + "' is not a string");
	auto st = v.s;
	strip(st);
	if (st.find(',') != std::string::npos)
		emsgroot("The expression '" + st + "' in '" + name + "' must not contain a comma");
	return st;
}

std::vector<double> InputNode::find_vector(const std::string &name)
{
	add_used(name);
	const Node &v = child(n(), name);
	if (v.kind != Node::ARRAY) throw std::runtime_error("'" + name + "' is not an array");
	std::vector<double> out;
	for (const auto &e : v.arr) out.push_back(as_number(*e));
	return out;
}

std::string InputNode::stringfield(string name, string em) { return stringfield(name.c_str(), em); }

std::string InputNode::stringfield(const char *name, string em)
{
	if (!contains(name)) {
		if (em == "") return "";
		emsgroot(em + " a value for '" + name + "' must be specified");
	}
	return stringfield_unchecked(name);
}

std::string InputNode::stringfield_allowcomma(string name, string em)
{
	return stringfield_allowcomma(name.c_str(), em);
}

std::string InputNode::stringfield_allowcomma(const char *name, string em)
{
	if (!contains(name)) {
		if (em == "") return "";
		emsgroot(em + " a value for '" + name + "' must be specified");
	}
	add_used(name);
	const Node &v = child(n(), name);
	if (v.kind != Node::STRING) throw std::runtime_error(std::string("'") + name + "' is not a string");
	auto st = v.s;
	strip(st);
	return st;
}

double InputNode::numberfield_unchecked(const std::string &name)
{
	return as_number(child(n(), name));
}

double InputNode::numberfield(const char *name, string em)
{
	if (!contains(name)) {
		if (em == "") return UNSET;
		emsgroot(em + " a value for '" + name + "' must be specified");
	}
	return numberfield_unchecked(name);
}

int InputNode::intfield_unchecked(const std::string &name)
{
	add_used(name);
	const Node &v = child(n(), name);
	if (v.kind != Node::INT) throw std::runtime_error("'" + name + "' is not an integer");
	return (int)v.i;
}

vector<string> InputNode::keys() const
{
	vector<string> k;
	for (const auto &p : n().tab) k.push_back(p.first);
	return k;
}

InputNode parsefile(const std::string &inputfilename)
{
	Node n = parse_toml_file(inputfilename);
	const Node *base = n.find("baseinputfile");
	if (base != nullptr) {
		if (base->kind != Node::STRING) throw std::runtime_error("baseinputfile must be a string");
		Node b = parse_toml_file(base->s);
		for (const auto &p : b.tab) {
			if (n.find(p.first) == nullptr) n.tab.push_back(p);
		}
	}
	return InputNode(n, "", NULL);
}
