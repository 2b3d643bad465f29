"""Logger with the reference's ``add_to_log`` contract (slowquant/logger.py:1-24)."""


class _Logger:
    def __init__(self) -> None:
        self.log = ""
        self.print_output = True
        self.print_warnings = True

    def add_to_log(self, content: str, is_warning: bool = False) -> None:
        content += "\n"
        if is_warning:
            content = f"WARNING: {content}"
        if self.print_output or (is_warning and self.print_warnings):
            print(content, end="")
        self.log += content
