/* project-written empty stand-in: the scanner path needs nothing from esl_getopts.h */
