import sys

from .create_rate_subs import main

sys.exit(main())
