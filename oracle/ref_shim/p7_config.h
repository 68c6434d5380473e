/* project-written empty stand-in: the scanner path needs nothing from p7_config.h */
