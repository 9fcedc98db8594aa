/* Stand-in for the header bison writes from the reference's VEX grammar
 * (sfxc/lib/vex_parser/vex_parser/src/vex_parser.yy, %defines "vex_parser.h"):
 * the grammar itself is restated in vex_grammar.cc, which needs no token
 * table from here.  Test infrastructure only. */
#ifndef SFXC_ORACLE_VEX_PARSER_H
#define SFXC_ORACLE_VEX_PARSER_H
#endif
