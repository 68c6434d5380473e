/* project-written stand-in for the generated config header */
#define INFERNAL_VERSION "1.1.5-shim"
#define INFERNAL_DATE    "shim"
